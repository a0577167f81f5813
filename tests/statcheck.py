"""Statistical parity helpers: compare two sets of independent Monte Carlo renders
(one per seed) of the same scene, pixel-block by pixel-block, at 3 sigma of the
combined standard error of the block means."""
import numpy as np


def block_sums(imgs, b):
    """imgs [K, S, H, W, 3] -> [K, S, H//b, W//b, 3] block sums (image cropped to a multiple of b)."""
    K, S, H, W, C = imgs.shape
    H2, W2 = (H // b) * b, (W // b) * b
    x = imgs[:, :, :H2, :W2].astype(np.float64)
    return x.reshape(K, S, H2 // b, b, W2 // b, b, C).sum(axis=(3, 5))


def zscores(a, b, block=4):
    """z per block and slot for run sets a [Ka,...] and b [Kb,...]."""
    A, B = block_sums(np.asarray(a), block), block_sums(np.asarray(b), block)
    ma, mb = A.mean(0), B.mean(0)
    va = A.var(0, ddof=1) / A.shape[0]
    vb = B.var(0, ddof=1) / B.shape[0]
    se = np.sqrt(va + vb)
    with np.errstate(divide="ignore", invalid="ignore"):
        z = np.where(se > 0, (ma - mb) / se, np.where(np.abs(ma - mb) > 1e-6 * (np.abs(ma) + np.abs(mb) + 1e-12), np.inf, 0.0))
    return z, ma, mb, se


def total_z(a, b):
    """z of the whole-image sum per slot and channel."""
    A = np.asarray(a, np.float64).sum(axis=(2, 3))
    B = np.asarray(b, np.float64).sum(axis=(2, 3))
    se = np.sqrt(A.var(0, ddof=1) / A.shape[0] + B.var(0, ddof=1) / B.shape[0])
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(se > 0, (A.mean(0) - B.mean(0)) / se, 0.0), A.mean(0), B.mean(0), se


def assert_parity(a, b, block=4, z_max=3.0, max_frac=0.03, total_max=4.0, slots=None, label=""):
    """Fail when more than max_frac of the non-empty blocks of any slot exceed z_max,
    or when the whole-image sum of a slot differs by more than total_max sigma."""
    z, ma, mb, se = zscores(a, b, block)
    tz, ta, tb, tse = total_z(a, b)
    S = z.shape[0]
    report = []
    ok = True
    for s in range(S) if slots is None else slots:
        zs = z[s]
        live = (se[s] > 0) | (np.abs(ma[s]) + np.abs(mb[s]) > 0)
        n = int(live.sum())
        frac = float((np.abs(zs[live]) > z_max).mean()) if n else 0.0
        worst_total = float(np.max(np.abs(tz[s])))
        report.append(f"{label} slot {s}: blocks={n} frac|z|>{z_max}={frac:.4f} total_z={np.round(tz[s], 2)} "
                      f"total_a={np.round(ta[s], 5)} total_b={np.round(tb[s], 5)}")
        if frac > max_frac or worst_total > total_max:
            ok = False
    msg = "\n".join(report)
    assert ok, msg
    return msg
