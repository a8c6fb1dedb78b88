"""Learned ELL-tile cost model: the float64 oracle, the GPU training and
inference kernels against it, and what the trained network gains over the
analytic model on held-out GB300 timings."""
import ctypes
import os

import numpy as np
import pytest

import oracle.mlp as O
from stile_gb300 import mlp_cost as MC

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DATA = os.path.join(ROOT, "stile_gb300", "gb300_ell_timings.npz")
MODEL = os.path.join(ROOT, "stile_gb300", "gb300_mlp_cost_model.json")


def _problem(n=300, seed=0):
    rng = np.random.default_rng(seed)
    p = MC.init_params(seed, 0.3).astype(np.float64)
    p += rng.normal(0, 0.05, p.size)
    x = rng.standard_normal((n, MC.FEATURES))
    t = rng.standard_normal(n)
    return p, x, t


def test_oracle_gradient_matches_finite_differences():
    p, x, t = _problem(40)
    _, g = O.loss_and_grad(p, x, t)
    rng = np.random.default_rng(3)
    for i in rng.choice(len(p), 40, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        fd = (O.loss_and_grad(p + e, x, t)[0] - O.loss_and_grad(p - e, x, t)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-7


def test_features_shape_and_meaning():
    rn = np.array([[4, 4, 0, 2], [1, 1, 1, 1]])
    f = MC.ell_tile_features(4, 4, rn, np.array([3, 4]), 128)
    assert f.shape == (2, MC.FEATURES)
    assert np.allclose(f[:, 2], [10 / 16, 4 / 16])      # density
    assert np.allclose(f[:, 10], [0.75, 1.0])           # non-empty rows
    assert np.allclose(f[:, 6], [3 / 10, 1.0])          # distinct / nnz


def test_learned_model_beats_analytic_on_held_out_timings():
    """On GB300 ELL-tile timings the networks never saw, the learned model's
    mean |log(predicted / measured)| is below the analytic fit's."""
    from stile_gb300.calibrate_mlp import split
    d = np.load(DATA)
    m = MC.MlpCostModel.from_json(open(MODEL).read())
    test = split(len(d["log_ms"]))
    for atomic, net in ((False, m.owned), (True, m.atomic)):
        sel = test & (d["atomic"] == atomic)
        assert sel.sum() >= 20
        pred = O.forward(net.params, net.standardise(d["features"][sel]))
        mlp_err = np.mean(np.abs(pred - d["log_ms"][sel]))
        ana_err = np.mean(np.abs(d["analytic_log_ms"][sel] - d["log_ms"][sel]))
        print(f"atomic={atomic}: held-out mean |log err| mlp {mlp_err:.3f} analytic {ana_err:.3f}")
        assert mlp_err < ana_err


def _gpu(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device="cuda")


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.gpu
def test_inference_kernel_matches_oracle():
    from stile_gb300 import _lib
    import torch
    lib = _lib.load()
    p, x, _ = _problem(1000, seed=1)
    y = torch.empty(len(x), device="cuda")
    pd, xd = _gpu(p), _gpu(x)  # kept alive until the kernel has run
    _lib.check(lib.stile_mlp_forward(pd.data_ptr(), xd.data_ptr(), len(x), y.data_ptr(), _stream()), "fwd")
    torch.cuda.synchronize()
    ref = O.forward(p.astype(np.float32), x.astype(np.float32))
    assert np.max(np.abs(y.cpu().numpy() - ref)) <= 1e-4 * max(1.0, np.abs(ref).max())


@pytest.mark.gpu
def test_gradient_kernels_match_oracle():
    from stile_gb300 import _lib
    import torch
    lib = _lib.load()
    p, x, t = _problem(300, seed=2)
    p32, x32, t32 = p.astype(np.float32), x.astype(np.float32), t.astype(np.float32)
    n = len(x)
    work = torch.empty(n * MC.WORK, device="cuda")
    dy = torch.empty(n, device="cuda")
    grad = torch.empty(MC.N_PARAMS, device="cuda")
    loss = torch.empty(1, device="cuda")
    pd, xd, td = _gpu(p32), _gpu(x32), _gpu(t32)  # kept alive until the kernels have run
    _lib.check(lib.stile_mlp_gradient(pd.data_ptr(), xd.data_ptr(), td.data_ptr(), n,
                                      work.data_ptr(), dy.data_ptr(), grad.data_ptr(), loss.data_ptr(), _stream()),
               "grad")
    torch.cuda.synchronize()
    ref_loss, ref_g = O.loss_and_grad(p32, x32, t32)
    g = grad.cpu().numpy()
    assert abs(loss.item() - ref_loss) <= 1e-4 * ref_loss
    assert np.linalg.norm(g - ref_g) <= 1e-4 * np.linalg.norm(ref_g)


@pytest.mark.gpu
def test_gpu_training_fits_a_smooth_target():
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (600, MC.FEATURES)).astype(np.float32)
    t = (np.sin(2 * x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] + 0.3 * x[:, 3]).astype(np.float32)
    net, hist = MC.train_net(x, t, epochs=1500, lr=3e-3, log_every=500)
    assert hist[-1][1] < 0.05 * hist[0][1]
    pred = O.forward(net.params, net.standardise(x))
    assert np.mean((pred - t) ** 2) < 0.02


@pytest.mark.gpu
def test_planner_with_learned_model_gives_a_correct_operator():
    import torch
    import oracle.semantics as S
    from stile_gb300 import synthetic as syn
    from stile_gb300.api import PlanConfig, SpmmOperator
    A = syn.community_graph(n=8192, target_nnz=60_000, seed=5)
    op = SpmmOperator(A, 128, PlanConfig(learned=True))
    assert "mlp" in op.plan.meta["cost_model"]
    B = np.random.default_rng(0).standard_normal((A.shape[1], 128)).astype(np.float32)
    C = op(torch.as_tensor(B, device="cuda")).cpu().numpy()
    assert S.rel_fro(C, S.spmm_fp64(A, B)) <= 1e-2
    assert op.handle.error_flag() == 0
