"""The collision-outcome surrogate: BF16 tensor-core MLP kernels checked
against the CPU oracle (oracle/mlp_oracle.py), training, the ensemble's
uncertainty, and a small end-to-end screened sweep that shows what the
network gains over simulating every point."""
import numpy as np
import pytest

from oracle import mlp_oracle
from spacelab_gb300 import batch as B
from spacelab_gb300 import surrogate as S
from spacelab_gb300 import sweep as W

pytestmark = pytest.mark.gpu

ARCH = dict(n_in=8, hidden=256, layers=4, n_out=4)


def _net(seed=1, max_batch=256):
    return S.Mlp(ARCH["n_in"], ARCH["n_out"], ARCH["hidden"], ARCH["layers"], max_batch=max_batch, seed=seed)


def _layer_slices():
    din, dout, offs, _ = mlp_oracle.layout(**ARCH)
    return [(w, w + a * b) for (w, _), a, b in zip(offs, din, dout)] + [(bo, bo + b) for (_, bo), b in zip(offs, dout)]


def test_mlp_forward_matches_cpu_oracle():
    """The forward pass (tcgen05 GEMMs) against the numpy oracle with the same
    bf16 rounding points: the two differ only in FP32 accumulation order,
    which can move an activation across a bf16 rounding boundary (one bf16
    ulp = 2^-8 relative); bar 5e-3 of the largest output (measured: 2.6e-4
    to 4.4e-3 over five seeds)."""
    net = _net()
    rng = np.random.default_rng(0)
    x = rng.normal(size=(100, 8)).astype(np.float32)
    y = net.predict(x)
    ref, *_ = mlp_oracle.forward(net.params(), x, **ARCH)
    scale = np.abs(ref).max()
    assert np.abs(y - ref).max() <= 5e-3 * scale


def test_mlp_gradients_match_cpu_oracle():
    """Every layer's weight and bias gradients against the oracle: within
    3e-3 of the layer's gradient norm (measured: at most 7.6e-4 over five
    seeds) and aligned to 1e-5 in cosine."""
    net = _net()
    rng = np.random.default_rng(1)
    x = rng.normal(size=(128, 8)).astype(np.float32)
    y = rng.normal(size=(128, 4)).astype(np.float32)
    loss, g = net.gradients(x, y)
    l_ref, g_ref = mlp_oracle.loss_and_grads(net.params(), x, y, **ARCH)
    assert abs(loss - l_ref) <= 1e-3 * l_ref
    for a, b in _layer_slices():
        gr, gg = g_ref[a:b], g[a:b]
        nr = np.linalg.norm(gr)
        if nr == 0:
            assert np.abs(gg).max() == 0
            continue
        assert np.linalg.norm(gg - gr) <= 3e-3 * nr, (a, b)
        assert gg @ gr / (np.linalg.norm(gg) * nr) > 1 - 1e-5


def test_mlp_learns_a_smooth_map():
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, size=(4096, 8)).astype(np.float32)
    y = np.stack([np.sin(2 * x[:, 0]) + x[:, 1] ** 2, x[:, 2] * x[:, 3], np.cos(x[:, 4] + x[:, 5]),
                  np.abs(x[:, 6]) - x[:, 7]], axis=1).astype(np.float32)
    net = _net(seed=3)
    curve = net.train(x, y, epochs=60, batch=256, lr=2e-3, seed=0)
    assert curve[-1] < curve[0] / 20
    xt = rng.uniform(-1, 1, size=(512, 8)).astype(np.float32)
    yt = np.stack([np.sin(2 * xt[:, 0]) + xt[:, 1] ** 2, xt[:, 2] * xt[:, 3], np.cos(xt[:, 4] + xt[:, 5]),
                   np.abs(xt[:, 6]) - xt[:, 7]], axis=1)
    assert np.mean((net.predict(xt) - yt) ** 2) < 0.05 * yt.var()


def test_ensemble_spread_grows_outside_the_data():
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, size=(2048, 8))
    y = np.stack([x[:, 0] + x[:, 1], x[:, 2] * 2, x[:, 3] ** 2, x[:, 4]], axis=1)
    ens = S.Ensemble(8, 4, members=5, seed=5)
    ens.fit(x, y, epochs=40, batch=256, lr=2e-3)
    _, s_in = ens.predict(rng.uniform(-1, 1, size=(256, 8)))
    _, s_out = ens.predict(rng.uniform(4, 6, size=(256, 8)))
    assert s_out.mean() > 3 * s_in.mean()


def test_screened_sweep_gains_over_simulating_every_point():
    """Small end to end: outcomes of 1280 simulated collisions (the batched
    solver's sweep recipe with 64-160-sphere targets, 3000 steps) train the
    ensemble on 1024 of them; the screening threshold comes from the other
    256 (mean absolute error of the accepted ones <= 0.8 of each outcome's
    spread -- a small training set gives a coarse surrogate); a 3000-point
    sweep is screened and its uncertain points and a 3% audit are re-run.
    The network must beat simulating every point on cost, and on the audit
    it must beat the method without it -- predicting the training mean --
    on every outcome that varies (on validation it was at 0.54-0.73 of the
    training mean's error for the three remnant outcomes and 0.13 for the
    dissipated fraction; with 16-40-sphere targets the outcomes are too
    erratic for 1024 collisions to teach)."""
    steps = 3000
    data = B.sample_collisions(1280, seed=11, nt_range=(64, 160), clearance=W.CLEARANCE, k_speed_div=W.K_SPEED_DIV)
    y, info = W.simulate(data, steps, mode="mixed_df")
    assert info["nonfinite"] == 0
    x = W.features(data)
    ens = S.Ensemble(8, 4, members=5, seed=9)
    ens.fit(x[:1024], y[:1024], epochs=150, batch=128, lr=1e-3)
    pick = W.pick_threshold(ens, x[1024:], y[1024:], error_target=0.8)
    assert pick["threshold"] > 0 and pick["accept_fraction"] > 0.2
    assert max(pick["mae_std_units"]) <= 0.8
    points = W.sample_params(3000, seed=12, nt_range=(64, 160))
    res = W.screen_sweep(ens, points, steps, threshold=pick["threshold"], audit=0.03, seed=13, sim_mode="mixed_df",
                         fp64_check=8)
    assert res["rerun"] < 0.7 * res["points"]
    assert res["cost_ratio"] > 1.3
    mae = np.array(res["audit_mae"])
    spread = np.array(res["outcome_std"])
    informative = spread > 1e-9
    # the method without the network, on the same audit points
    mean_only = np.array(res["audit_mae_training_mean"])
    assert np.all(mae[informative] < mean_only[informative]), (mae, mean_only)
    # the mixed re-runs stand for the FP64 method: their outcomes agree to a
    # small part of each outcome's spread
    d = np.array(res["fp64_check"]["mean_abs_diff"])
    assert np.all(d[informative] <= 0.2 * spread[informative])


def _bf16_bits(x: np.ndarray) -> np.ndarray:
    """float32 -> bf16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def _bf16_to_f32(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)


def _diag_gemm(A, B, bias, act, kernel):
    import ctypes
    from spacelab_gb300 import _lib
    M, K = A.shape
    N = B.shape[0]
    C = np.zeros((M, N), dtype=np.float32)
    Cb = np.zeros((M, N), dtype=np.uint16)
    u16 = ctypes.POINTER(ctypes.c_uint16)
    f32 = ctypes.POINTER(ctypes.c_float)
    rc = _lib.lib().sl_diag_gemm_bf16(M, N, K, A.ctypes.data_as(u16), B.ctypes.data_as(u16),
                                      bias.ctypes.data_as(f32), act, kernel, C.ctypes.data_as(f32),
                                      Cb.ctypes.data_as(u16))
    assert rc == 0, _lib.lib().sl_last_error()
    return C, Cb


@pytest.mark.parametrize("M,N,K", [(128, 256, 256), (256, 256, 32), (100, 32, 256), (256, 256, 1024),
                                   (37, 256, 64), (1000, 128, 256), (300, 64, 96), (1024, 32, 256)])
def test_tcgen05_gemm_matches_the_product(M, N, K):
    """The tcgen05/TMEM GEMM (kernel 1) on bf16 inputs against the exact
    product of the same bf16 values (float64), and against the mma.sync
    kernel (0) where K allows it.  Bar: each entry within 2e-6 of the sum of
    its terms' magnitudes (FP32 accumulation of K products); the bf16 GELU
    output within one bf16 ulp of the rounded exact value."""
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = _bf16_bits(rng.normal(size=(M, K)).astype(np.float32))
    B = _bf16_bits(rng.normal(size=(N, K)).astype(np.float32) * 0.1)
    bias = rng.normal(size=N).astype(np.float32)
    Af, Bf = _bf16_to_f32(A).astype(np.float64), _bf16_to_f32(B).astype(np.float64)
    ref = Af @ Bf.T + bias
    mag = np.abs(Af) @ np.abs(Bf).T + np.abs(bias)
    C, Cb = _diag_gemm(A, B, bias, 1, kernel=1)
    assert np.all(np.abs(C - ref) <= 2e-6 * mag)
    gelu = 0.5 * ref * (1.0 + np.vectorize(__import__("math").erf)(ref / np.sqrt(2.0)))
    ulp = np.abs(_bf16_to_f32(_bf16_bits(gelu.astype(np.float32)))) * 2.0 ** -7 + 1e-30
    assert np.all(np.abs(_bf16_to_f32(Cb) - gelu) <= ulp + 2e-6 * mag)
    if K % 32 == 0:
        C0, _ = _diag_gemm(A, B, bias, 1, kernel=0)
        assert np.all(np.abs(C - C0) <= 4e-6 * mag)
