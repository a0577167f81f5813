"""Host-side statistics of the bench line (no GPU): the gradient error against a high-spp
reference with the Monte Carlo noise of both sides taken out of the bias, and the workload
config both arms print."""
import numpy as np

import bench


def _runs(rng, g, runs, sd, bias=0.0):
    return g + bias + rng.normal(0.0, sd, size=(runs, g.size))


def test_rmse_summary_unbiased_runs_have_no_excess_bias():
    rng = np.random.default_rng(0)
    g = rng.normal(size=200)
    run_spp, ref_spp, sd = 16, 1024, 0.5
    G = _runs(rng, g, 16, sd)
    g_ref = g + rng.normal(0.0, sd * np.sqrt(run_spp / ref_spp), size=g.size)
    r = bench.rmse_summary(G, run_spp, g_ref, ref_spp)
    assert 0.3 < r["diff_over_noise"] < 3.0          # the difference is what the noise predicts
    assert r["rel_bias_excess"] < 0.5 * r["rel_diff"]
    assert r["spp_to_1pct_with_bias"] >= r["spp_to_1pct_variance_only"]
    # spp to 1%: run_spp * tr Cov / (1e-4 |g|^2)
    tr = G.var(0, ddof=1).sum()
    assert np.isclose(r["spp_to_1pct_variance_only"], run_spp * tr / (1e-4 * (g_ref @ g_ref)))


def test_rmse_summary_detects_a_real_bias():
    rng = np.random.default_rng(1)
    g = rng.normal(size=200)
    run_spp, ref_spp, sd = 16, 4096, 0.05
    G = _runs(rng, g, 64, sd, bias=0.05)               # a shift of 0.05 per coordinate
    g_ref = g + rng.normal(0.0, sd * np.sqrt(run_spp / ref_spp), size=g.size)
    r = bench.rmse_summary(G, run_spp, g_ref, ref_spp)
    assert r["diff_over_noise"] > 10.0
    expected = 0.05 * np.sqrt(g.size) / np.linalg.norm(g_ref)
    assert abs(r["rel_bias_excess"] - expected) < 0.2 * expected
    # a bias above 1% of |g| can never be averaged away
    assert r["spp_to_1pct_with_bias"] == float("inf")


def test_both_arms_print_the_same_config():
    for name in bench.WORKLOADS:
        a = bench.workload_config(name, 1)
        b = bench.workload_config(name, 1, bench.build_spec(name))
        assert a == b
        assert a["parallelism"] == "replicas x1" and a["spp"] == bench.WORKLOADS[name]["spp"]
