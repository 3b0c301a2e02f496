"""The learned-radius network's CPU restatement (oracle/radius_mlp.py): the
bfloat16 rounding it emulates and a finite-difference check of its analytic
gradient, which then checks the GPU backward kernels."""
import numpy as np

from oracle import radius_mlp as R


def test_bf16_rounding_known_answers():
    x = np.array([1.0, 1.0 + 2.0**-8, 1.0 + 3 * 2.0**-8, -1.0 - 2.0**-8, 1.0 + 2.0**-7,
                  3.0e38, 0.0, -2.5], dtype=np.float32)
    want = np.array([1.0, 1.0, 1.0 + 2.0**-6, -1.0, 1.0 + 2.0**-7, 0.0, 0.0, -2.5],
                    dtype=np.float32)
    got = R.bf16(x)
    assert np.array_equal(got[:5], want[:5]) and got[6] == 0.0 and got[7] == -2.5
    assert np.isfinite(got[5])  # below the largest bfloat16 (about 3.39e38)


def test_layout_matches_engine_header():
    assert R.N_PARAMS == 64 * 11 + 64 + 64 * 64 + 64 + 64 + 1 + 11 + 11
    assert R.N_TRAINED == R.N_PARAMS - 22


def _params(rng):
    p = np.zeros(R.N_PARAMS, np.float32)
    p[: R.N_TRAINED] = rng.normal(0, 0.3, R.N_TRAINED)
    a, b = R.LAYOUT["sigma"]
    p[a:b] = rng.uniform(0.5, 2.0, b - a)
    a, b = R.LAYOUT["mu"]
    p[a:b] = rng.normal(0, 0.5, b - a)
    return p


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = _params(rng)
    feat = rng.normal(0, 1, (64, R.N_FEATURES)).astype(np.float32)
    tgt = rng.normal(0, 1, 64).astype(np.float32)
    rows = np.arange(64)
    g, loss = R.gradient(p, feat, tgt, rows, bf=False)
    assert np.isfinite(loss) and loss > 0
    idx = rng.choice(R.N_TRAINED, 60, replace=False)
    for i in idx:
        h = 1e-3 * max(1.0, abs(float(p[i])))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        hh = (float(pp[i]) - float(pm[i])) / 2
        fd = (R.gradient(pp, feat, tgt, rows, bf=False)[1]
              - R.gradient(pm, feat, tgt, rows, bf=False)[1]) / (2 * hh)
        assert abs(fd - g[i]) <= 2e-3 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_bf16_forward_close_to_exact():
    rng = np.random.default_rng(1)
    p = _params(rng)
    feat = rng.normal(0, 1, (256, R.N_FEATURES)).astype(np.float32)
    y_bf, _ = R.forward(p, feat, bf=True)
    y_ex, _ = R.forward(p, feat, bf=False)
    assert np.max(np.abs(y_bf - y_ex)) < 0.05 * max(1.0, np.max(np.abs(y_ex)))


def test_engine_layout_matches_oracle():
    """The Python model's parameter layout is the oracle's (and the kernels')."""
    from fast_hdbscan_gb300 import radius

    assert radius.N_PARAMS == R.N_PARAMS and radius.N_TRAINED == R.N_TRAINED
    assert radius.LAYOUT == R.LAYOUT
