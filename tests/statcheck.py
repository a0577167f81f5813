"""Statistical parity helpers: compare two sets of independent Monte Carlo renders
(one per seed) of the same scene, pixel-block by pixel-block, at 3 sigma of the
combined standard error of the block means.

Under the null hypothesis (same expectation) each block's z is Student-t distributed
with the Welch-Satterthwaite degrees of freedom, so a fraction p0 = P(|t| > 3) of the
blocks exceeds 3 by chance (0.27% for normal z, about 0.6% at 16 + 16 runs). The
allowance for a slot with n blocks is the count that a Binomial(n, p0) exceeds with
probability below `alpha` (1e-3 per slot): a correct renderer fails a slot about once
in a thousand checks, a biased one in most.

Edge-sampled derivative estimates are heavy-tailed: with few runs their sample variance is
often too small and the t test too wide. The runs of each side are therefore grouped into
`batches` batch means (consecutive runs averaged) before the test, so that each tested
value is itself an average of many paths and close to normal; more runs per side then
tighten the test instead of exposing the tails."""
import numpy as np

MIN_RUNS = 16
BATCHES = 16


def batch_means(x, batches=BATCHES):
    """[K, ...] runs -> [batches, ...] means of consecutive groups (unchanged when K <= batches)."""
    x = np.asarray(x)
    K = x.shape[0]
    if K <= batches:
        return x
    m = K // batches
    return x[: m * batches].astype(np.float64).reshape((batches, m) + x.shape[1:]).mean(axis=1)


def block_sums(imgs, b):
    """imgs [K, S, H, W, 3] -> [K, S, H//b, W//b, 3] block sums (image cropped to a multiple of b)."""
    K, S, H, W, C = imgs.shape
    H2, W2 = (H // b) * b, (W // b) * b
    x = imgs[:, :, :H2, :W2].astype(np.float64)
    return x.reshape(K, S, H2 // b, b, W2 // b, b, C).sum(axis=(3, 5))


def zscores(a, b, block=4):
    """z per block and slot for run sets a [Ka,...] and b [Kb,...], and the Welch
    degrees of freedom per block."""
    A, B = block_sums(np.asarray(a), block), block_sums(np.asarray(b), block)
    ma, mb = A.mean(0), B.mean(0)
    va = A.var(0, ddof=1) / A.shape[0]
    vb = B.var(0, ddof=1) / B.shape[0]
    se = np.sqrt(va + vb)
    with np.errstate(divide="ignore", invalid="ignore"):
        z = np.where(se > 0, (ma - mb) / se, np.where(np.abs(ma - mb) > 1e-6 * (np.abs(ma) + np.abs(mb) + 1e-12), np.inf, 0.0))
        df = np.where(se > 0, (va + vb) ** 2 / (va ** 2 / max(A.shape[0] - 1, 1) + vb ** 2 / max(B.shape[0] - 1, 1)),
                      np.inf)
    return z, ma, mb, se, df


def total_z(a, b):
    """z of the whole-image sum per slot and channel."""
    A = np.asarray(a, np.float64).sum(axis=(2, 3))
    B = np.asarray(b, np.float64).sum(axis=(2, 3))
    se = np.sqrt(A.var(0, ddof=1) / A.shape[0] + B.var(0, ddof=1) / B.shape[0])
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(se > 0, (A.mean(0) - B.mean(0)) / se, 0.0), A.mean(0), B.mean(0), se


def allowed_exceedances(n, p0, alpha=1e-3):
    """Smallest k with P(Binomial(n, p0) > k) < alpha."""
    from scipy import stats
    return int(stats.binom.ppf(1.0 - alpha, n, p0)) if n else 0


def null_exceedance_prob(df, z_max=3.0):
    """Mean over blocks of P(|t_df| > z_max): the expected fraction of blocks beyond z_max
    for a correct renderer."""
    from scipy import stats
    df = np.asarray(df, np.float64)
    df = np.where(np.isfinite(df), np.maximum(df, 1.0), 1e6)
    return float(np.mean(2.0 * stats.t.sf(z_max, df))) if df.size else 0.0


def assert_parity(a, b, block=4, z_max=3.0, alpha=1e-3, total_max=4.0, slots=None, label="", min_runs=MIN_RUNS,
                  batches=BATCHES):
    """Fail when, in any slot, more non-empty blocks exceed z_max than the binomial allowance
    (null fraction from the t distribution, false-alarm rate alpha per slot), or when the
    whole-image sum of a slot differs by more than total_max sigma. Each side's runs are
    first reduced to `batches` batch means."""
    assert len(a) >= min_runs and len(b) >= min_runs, f"{label}: need >= {min_runs} runs per side"
    a, b = batch_means(a, batches), batch_means(b, batches)
    z, ma, mb, se, df = zscores(a, b, block)
    tz, ta, tb, tse = total_z(a, b)
    S = z.shape[0]
    report = []
    ok = True
    for s in range(S) if slots is None else slots:
        zs = z[s]
        live = (se[s] > 0) | (np.abs(ma[s]) + np.abs(mb[s]) > 0)
        n = int(live.sum())
        nbad = int((np.abs(zs[live]) > z_max).sum())
        p0 = null_exceedance_prob(df[s][live], z_max)
        allow = allowed_exceedances(n, p0, alpha)
        worst_total = float(np.max(np.abs(tz[s])))
        report.append(f"{label} slot {s}: blocks={n} |z|>{z_max}: {nbad} (null rate {p0:.4f}, allowed {allow}) "
                      f"total_z={np.round(tz[s], 2)} total_a={np.round(ta[s], 5)} total_b={np.round(tb[s], 5)}")
        if nbad > allow or worst_total > total_max:
            ok = False
    msg = "\n".join(report)
    assert ok, msg
    return msg


def image_mean_rel_error(g, c):
    """|sum(g) - sum(c)| / |sum(c)| over the image slot (the relative error of the image mean)."""
    g, c = np.asarray(g, np.float64), np.asarray(c, np.float64)
    return float(abs(g.sum() - c.sum()) / abs(c.sum()))


def rel_l1(g, c):
    """sum |g - c| / sum |c| (per-pixel relative L1 error, noise included)."""
    g, c = np.asarray(g, np.float64), np.asarray(c, np.float64)
    return float(np.abs(g - c).sum() / np.abs(c).sum())
