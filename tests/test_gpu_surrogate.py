"""Learned source-term surrogate on the GPU against its CPU oracle
(oracle/mlp_oracle.py), through the C ABI.

  * the tcgen05 GEMM against an f64 product of the same bf16 operands;
  * the surrogate's input rows against the oracle's features of the state
    read back from the model;
  * the forward pass and the loss gradient against the oracle, which rounds
    to bf16 at the same points as the GPU (tolerances below);
  * training on pairs captured from the plain model lowers the loss, and a
    run with the trained network is closer to the plain model than a run
    with the untrained network (the method without training).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mo():
    from oracle import mlp_oracle

    return mlp_oracle


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 256, 192), (1000, 1344, 512), (4096, 512, 1344),
                                   (20480, 256, 128), (3328, 1344, 512), (40000, 512, 1344)])
def test_gemm_bf16(lib_built, mo, M, N, K):
    """Both tile widths: 128-wide tiles for launches with fewer 256-wide
    tiles than SMs (the first four shapes), 256-wide ones otherwise (an
    N tail of 64 columns in 3328 x 1344; several tiles per CTA and both
    TMEM accumulators in turn in 40000 x 512)."""
    U = lib_built
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    C = U.gemm_bf16(mo.bf16_bits(A), mo.bf16_bits(B))
    ref = mo.bf16(A).astype(np.float64) @ mo.bf16(B).astype(np.float64).T
    # f32 accumulation of K exact bf16 products
    assert np.abs(C - ref).max() <= 1e-5 * np.abs(ref).max() * np.sqrt(K / 64.0) + 1e-6


def _batch(mo, n, seed):
    rng = np.random.default_rng(seed)
    X = np.zeros((n, mo.FPAD), np.float32)
    X[:, :1332 + mo.NEXTRA] = rng.standard_normal((n, 1332 + mo.NEXTRA)).astype(np.float32)
    T = np.zeros((n, mo.FPAD), np.float32)
    T[:, :1332] = 0.3 * rng.standard_normal((n, 1332)).astype(np.float32)
    return X, T


def test_forward_matches_oracle(lib_built, mo):
    U = lib_built
    U.surrogate_init(37, 36, seed=5)
    w = U.surrogate_get_params()
    # a larger output layer than the initial one, so the outputs are O(1)
    w[mo.OFF_W3:mo.OFF_B3] *= 10.0
    U.surrogate_set_params(w)
    X, _ = _batch(mo, 384, 1)
    Y = U.surrogate_forward(X)
    Yo, _ = mo.forward(w, X)
    # bf16 hidden activations: a last-place difference in an f32 sum can flip
    # one bf16 rounding, so compare in norm (and bound the worst element)
    rel = np.linalg.norm(Y - Yo) / np.linalg.norm(Yo)
    assert rel < 2e-3, rel
    assert np.abs(Y - Yo).max() < 2e-2 * np.abs(Yo).max()


@pytest.mark.parametrize("weighted", [False, True])
def test_gradient_matches_oracle(lib_built, mo, weighted):
    U = lib_built
    U.surrogate_init(37, 36, seed=7)
    U.set_option("surrogate_loss_weight", 1 if weighted else 0)
    w = U.surrogate_get_params()
    w[mo.OFF_W3:mo.OFF_B3] *= 10.0
    U.surrogate_set_params(w)
    X, T = _batch(mo, 256, 2)
    loss, g = U.surrogate_grad(X, T)
    U.set_option("surrogate_loss_weight", 0)
    lo, go = mo.loss_and_grad(w, X, T, 1332, weighted)
    assert abs(loss - lo) <= 1e-3 * lo
    for name, a, b in (("W1", mo.OFF_W1, mo.OFF_B1), ("b1", mo.OFF_B1, mo.OFF_W2), ("W2", mo.OFF_W2, mo.OFF_B2),
                       ("b2", mo.OFF_B2, mo.OFF_W3), ("W3", mo.OFF_W3, mo.OFF_B3), ("b3", mo.OFF_B3, mo.NPARAM)):
        rel = np.linalg.norm(g[a:b] - go[a:b]) / np.linalg.norm(go[a:b])
        assert rel < 2e-2, (name, rel)


def test_features_match_oracle(lib_built, mo):
    from umwm_gb300 import configs

    U = lib_built
    case = configs.hurricane(mm=40, nm=36, hours=1, dx=4000.0, dtg=600, seed=3)
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    U.set_option("max_substeps", 3)
    U.umwm_run(case.start, case.stop)
    Xg = U.surrogate_features()
    F, ust = U.get_state()
    im = F.shape[0]
    g = {k: U.get_field(k)[:im] for k in ("wdir", "wspd", "uc", "vc", "rhorat", "fice")}
    Xo, _ = mo.features(F, g["wdir"].astype(np.float64), g["wspd"], ust, U.get_field("d")[:im], U.get_field("dts"),
                        g["uc"], g["vc"], g["rhorat"], g["fice"], U.get_field("th").astype(np.float64),
                        float(U.get_field("dth")))
    U.umwm_finalize()
    # the GPU rounds its f32 feature to bf16: one bf16 step apart at most
    tol = np.abs(Xo) * 2.0 ** -7 + 1e-6
    bad = np.abs(Xg - Xo) > tol
    assert bad.mean() < 1e-4, (bad.sum(), np.argwhere(bad)[:5])


def test_training_and_surrogate_run(lib_built):
    """Pairs from a plain run of one random field train the network; pairs
    from another seed are held out.  On the held-out pairs the trained
    network's loss is well below the untrained network's (whose near-zero
    output is the step without a source term).  Ten substeps with the trained
    network and the energy-budget fallback keep the state finite and
    non-negative, and count every wet point once per substep."""
    from umwm_gb300 import configs

    U = lib_built
    train_case = configs.random_field(mm=64, nm=56, hours=3, dx=2000.0, seed=4)
    held_case = configs.random_field(mm=64, nm=56, hours=1, dx=2000.0, seed=5)
    U.surrogate_init(37, 36, seed=11)
    w0 = U.surrogate_get_params()
    U.surrogate_capture(300000, 1024)
    counts = []
    for case in (train_case, held_case):
        U.clear_inputs()
        case.stage(U)
        U.umwm_initialize(nml_text=case.nml)
        U.umwm_run(case.start, case.stop)
        U.umwm_finalize()
        counts.append(int(U.stat("surrogate_pairs")))
    U.surrogate_capture(0, 0)
    n_train, n_all = counts
    assert n_train > 50000 and n_all - n_train > 10000
    U.set_option("surrogate_holdout", n_all - n_train)
    loss_untrained = U.surrogate_eval(n_train, n_all - n_train)
    losses = U.surrogate_train(600, batch=1024, lr=1e-3, seed=1)
    U.set_option("surrogate_holdout", 0)
    assert np.isfinite(losses).all()
    assert losses[-20:].mean() < 0.5 * losses[:20].mean(), (losses[:5], losses[-5:])
    loss_trained = U.surrogate_eval(n_train, n_all - n_train)
    assert loss_trained < 0.5 * loss_untrained, (loss_trained, loss_untrained)

    U.clear_inputs()
    held_case.stage(U)
    U.umwm_initialize(nml_text=held_case.nml)
    U.set_option("surrogate", 1)
    U.set_option("max_substeps", 10)
    p0, f0 = U.stat("surrogate_points"), U.stat("surrogate_fallback")
    U.umwm_run(held_case.start, held_case.stop)
    pts, fb = U.stat("surrogate_points") - p0, U.stat("surrogate_fallback") - f0
    F, u = U.get_state()
    U.set_option("surrogate", 0)
    U.umwm_finalize()
    assert pts == 10 * F.shape[0] and 0 <= fb <= pts
    assert np.isfinite(F).all() and (F >= 0).all() and np.isfinite(u).all()


def test_all_fallback_is_the_plain_path(lib_built):
    """With a zero energy-budget tolerance every point falls back to the
    plain integration: the run must be bit-identical to a plain run."""
    from umwm_gb300 import configs

    U = lib_built
    case = configs.random_field(mm=64, nm=56, hours=3, dx=2000.0, seed=4)
    U.surrogate_init(37, 36, seed=11)

    def run(sur):
        U.clear_inputs()
        case.stage(U)
        U.umwm_initialize(nml_text=case.nml)
        U.set_option("max_substeps", 6)
        U.set_option("surrogate", 1 if sur else 0)
        U.set_option("surrogate_tol", 1e-30)
        U.umwm_run(case.start, case.stop)
        F, u = U.get_state()
        U.set_option("surrogate", 0)
        U.set_option("surrogate_tol", 0.1)
        U.umwm_finalize()
        return F, u

    Fp, up = run(False)
    p0, f0 = U.stat("surrogate_points"), U.stat("surrogate_fallback")
    Fs, us = run(True)
    assert U.stat("surrogate_fallback") - f0 == U.stat("surrogate_points") - p0 > 0
    np.testing.assert_array_equal(Fs, Fp)
    np.testing.assert_array_equal(us, up)
