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
    """exg_dg_features / exg_dg_ls_step against NumPy: feature scaling (own RMS, or the correction
    scale for the second difference), the one- and two-direction least-squares steps and the fallback
    (no decrease: x = base)."""
    torch = require_gpu()
    rng = np.random.default_rng(7)
    dpc, nc = 27, 150
    n = dpc * nc
    p0, p1, p2, r = (rng.normal(0, s, n) for s in (1.0, 0.9, 0.8, 1e-3))
    dev = [torch.tensor(v, device="cuda") for v in (p0, p1, p2, r)]
    feats = [p0, p0 - p1, p0 - 2 * p1 + p2, r]
    for diff_scale in (0.0, 0.37):
        x = torch.empty((4 * dpc, nc), dtype=torch.float32, device="cuda")
        rms = torch.empty(4, dtype=torch.float64, device="cuda")
        E._check(E._lib.exg_dg_features(*(E._ptr(v) for v in dev), dpc, nc, diff_scale, E._ptr(x), E._ptr(rms),
                                        E._stream()))
        sc = np.array([np.sqrt(np.mean(f * f)) for f in feats])
        if diff_scale > 0:
            sc[2] = diff_scale
        assert np.allclose(rms.cpu().numpy(), sc, rtol=1e-12)
        x_ref = np.concatenate([(f / s).reshape(nc, dpc).T for f, s in zip(feats, sc)], axis=0)
        assert np.allclose(x.cpu().numpy(), x_ref, rtol=1e-6, atol=1e-6)
    base = rng.normal(0, 1, n)

    def run(e, ae, f=None, af=None):
        out = torch.empty(n, dtype=torch.float64, device="cuda")
        stats = torch.empty(6, dtype=torch.float64, device="cuda")
        keep = [torch.tensor(v, device="cuda") if v is not None else None for v in (r, ae, e, af, f, base)]
        ptrs = [None if v is None else E._ptr(v) for v in keep]
        E._check(E._lib.exg_dg_ls_step(*ptrs, n, E._ptr(out), E._ptr(stats), E._stream()))
        return out.cpu().numpy(), stats.cpu().numpy()

    # one direction
    e = rng.normal(0, 1, n)
    ae = 0.5 * r + 1e-4 * rng.normal(0, 1, n)
    out, st = run(e, ae)
    c = float(r @ ae) / float(ae @ ae)
    assert np.allclose(st[:3], [r @ ae, ae @ ae, r @ r], rtol=1e-12)
    assert st[3] == pytest.approx(c, rel=1e-12) and st[4] == 0.0
    assert np.allclose(out, base + c * e, rtol=1e-14, atol=1e-14)
    # two directions: the normal equations
    f = rng.normal(0, 1, n)
    af = 0.3 * r + 2e-4 * rng.normal(0, 1, n)
    out, st = run(e, ae, f, af)
    M = np.array([[ae @ ae, ae @ af], [ae @ af, af @ af]])
    ce, cf = np.linalg.solve(M, [r @ ae, r @ af])
    assert st[3] == pytest.approx(ce, rel=1e-9) and st[4] == pytest.approx(cf, rel=1e-9)
    res = r - ce * ae - cf * af
    assert st[5] == pytest.approx(r @ r - res @ res, rel=1e-9)
    assert np.allclose(out, base + ce * e + cf * f, rtol=1e-12, atol=1e-12)
    # fallback: a correction orthogonal to the residual changes nothing
    ao = rng.normal(0, 1, n)
    ao -= (ao @ r) / (r @ r) * r
    out, st = run(e, ao)
    assert st[3] == 0.0 and st[4] == 0.0 and np.array_equal(out, base)


def test_pressure_sequence_checkpoint_restart(tmp_path):
    """Save after 20 steps, continue; a fresh sequence loaded from the file continues the same way
    (history, weights, Adam moments and step, training buffer restored; the multigrid's coarse
    warm start is not part of the state, so solutions agree to the solver tolerance)."""
    torch = require_gpu()
    from exadg_gb300 import learned_guess as LG

    rhs, _ = LG.tgv_rhs_sequence(30, n_cells=8, degree=2, modes=32)
    kw = dict(n_cells=8, degree=2, mode="learned", train_every=10, epochs=10)
    a = LG.PressureSequence(**kw)
    for b in rhs[:20]:
        a.step(b)
    path = str(tmp_path / "seq.bin")
    a.save(path)
    n_samples, trained = len(a.samples), a.trained
    ref = [a.step(b) for b in rhs[20:]]
    c = LG.PressureSequence(**kw)
    c.load(path)
    assert c.steps_done == 20 and c.trained == trained and len(c.samples) == n_samples
    out = [c.step(b) for b in rhs[20:]]
    for (xa, ra), (xc, rc) in zip(ref, out):
        assert abs(ra["iterations"] - rc["iterations"]) <= 1
        assert float(torch.linalg.norm(xa - xc)) <= 1e-7 * float(torch.linalg.norm(xa))
    wrong = LG.PressureSequence(n_cells=6, degree=2, mode="learned")
    with pytest.raises(ValueError):
        wrong.load(path)
