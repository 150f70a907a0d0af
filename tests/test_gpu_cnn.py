"""GPU parity of the hand-written CNN kernels (forward, parameter gradients) against the NumPy
oracle, and the learned-guess pipeline on a short pressure-Poisson sequence."""
import numpy as np
import pytest

import exadg_gb300 as E
from oracle import cnn_oracle as C
from tests.gpu_common import require_gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(4, 3, 5), (6, 6, 6)])
def test_cnn_forward_and_gradients(dims):
    torch = require_gpu()
    from exadg_gb300.cnn import CellPatchCNN

    ci, ch, co = 108, 32, 27
    net = CellPatchCNN(dims, ci, ch, co, seed=3)
    nc = int(np.prod(dims))
    rng = np.random.default_rng(0)
    x = rng.normal(0, 1, (ci, nc)).astype(np.float32)
    gy = rng.normal(0, 1, (co, nc)).astype(np.float32)
    p = net.params.cpu().numpy().astype(np.float64)
    xd = torch.tensor(x, device="cuda")
    y = net.forward(xd).cpu().numpy()
    y_ref, _ = C.forward(p, x.astype(np.float64), dims, ci, ch, co)
    assert np.linalg.norm(y - y_ref) <= 1e-5 * np.linalg.norm(y_ref)
    g = net.backward(xd, torch.tensor(gy, device="cuda")).cpu().numpy()
    g_ref = C.backward(p, x.astype(np.float64), gy.astype(np.float64), dims, ci, ch, co)
    o = 0
    for name, shape in net.layer_shapes():
        n = int(np.prod(shape))
        a, b = g[o:o + n], g_ref[o:o + n]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b) + 1e-6, name
        o += n


def test_cnn_training_reduces_loss():
    torch = require_gpu()
    from exadg_gb300.cnn import CellPatchCNN

    dims = (6, 6, 6)
    net = CellPatchCNN(dims, 8, 16, 4, seed=5)
    nc = 216
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn((8, nc), device="cuda", generator=g)
    target = 0.5 * x[:4].clone()
    l0 = net.train_step(x, target, lr=3e-3)
    for _ in range(200):
        l1 = net.train_step(x, target, lr=3e-3)
    assert l1 < 0.2 * l0


def test_learned_guess_sequence_small():
    torch = require_gpu()
    import math

    from exadg_gb300 import learned_guess as LG

    rhs, dt = LG.tgv_rhs_sequence(40, n_cells=8, degree=2, modes=32)
    ext = LG.PressureSequence(n_cells=8, degree=2, mode="extrapolation")
    lrn = LG.PressureSequence(n_cells=8, degree=2, mode="learned", train_every=10, epochs=30)
    for b in rhs:
        xe, re_ = ext.step(b)
        xl, rl = lrn.step(b)
        # both seedings reach the same (zero-mean) solution
        assert float(torch.linalg.norm(xe - xl)) <= 1e-6 * float(torch.linalg.norm(xe)) + 1e-12
    # the fallback rule guarantees the initial residual is never worse than extrapolation
    for r in lrn.log:
        if "r_ext_rel" in r:
            assert r["r0_rel"] <= r["r_ext_rel"] * (1 + 1e-9)
    assert any(r["source"] in ("learned", "fallback") for r in lrn.log)


def test_features_and_ls_step_on_device():
    """exg_dg_features / exg_dg_ls_step against NumPy: feature scaling by RMS, the least-squares step
    c = max(r.Ae / Ae.Ae, 0) and the fallback (c = 0, x = base) when the correction points uphill."""
    torch = require_gpu()
    rng = np.random.default_rng(7)
    dpc, nc = 27, 150
    n = dpc * nc
    p0, p1, p2, r = (rng.normal(0, s, n) for s in (1.0, 0.9, 0.8, 1e-3))
    dev = [torch.tensor(v, device="cuda") for v in (p0, p1, p2, r)]
    x = torch.empty((4 * dpc, nc), dtype=torch.float32, device="cuda")
    rms = torch.empty(4, dtype=torch.float64, device="cuda")
    E._check(E._lib.exg_dg_features(*(E._ptr(v) for v in dev), dpc, nc, E._ptr(x), E._ptr(rms), E._stream()))
    feats = [p0, p0 - p1, p0 - 2 * p1 + p2, r]
    rms_ref = np.array([np.sqrt(np.mean(f * f)) for f in feats])
    assert np.allclose(rms.cpu().numpy(), rms_ref, rtol=1e-12)
    x_ref = np.concatenate([(f / s).reshape(nc, dpc).T for f, s in zip(feats, rms_ref)], axis=0)
    assert np.allclose(x.cpu().numpy(), x_ref, rtol=1e-6, atol=1e-6)
    base = rng.normal(0, 1, n)
    for sign in (1.0, -1.0):
        e = rng.normal(0, 1, n)
        ae = sign * (0.5 * r + 0.1 * rng.normal(0, 1e-3, n))
        out = torch.empty(n, dtype=torch.float64, device="cuda")
        stats = torch.empty(4, dtype=torch.float64, device="cuda")
        td = [torch.tensor(v, device="cuda") for v in (r, ae, e, base)]
        E._check(E._lib.exg_dg_ls_step(*(E._ptr(v) for v in td), n, E._ptr(out), E._ptr(stats), E._stream()))
        c = max(float(r @ ae) / float(ae @ ae), 0.0)
        st = stats.cpu().numpy()
        assert np.allclose(st[:3], [r @ ae, ae @ ae, r @ r], rtol=1e-12)
        assert st[3] == pytest.approx(c, rel=1e-12, abs=0.0)
        assert (c > 0) == (sign > 0)
        assert np.allclose(out.cpu().numpy(), base + c * e, rtol=1e-14, atol=1e-14)
