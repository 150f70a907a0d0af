"""Learned initial guess for the sequence of pressure-Poisson solves (row a20).

ExaDG seeds every pressure solve of the dual-splitting scheme with the polynomial extrapolation
p0 = sum_i beta_i p^{n-i}, beta = (2, -1) for BDF2 (time_int_bdf_dual_splitting.cpp:489-498,
time_integration/extrapolation_constants.cpp:55-80).  Here a cell-patch CNN (csrc/cnn.cu) predicts a
correction to that extrapolation from, per cell, the DG coefficients of the last three pressures
(p^n and its first and second backward differences) and of the current right-hand side (entering as
the residual of the extrapolation, b - A p_ext).  It is trained online on the solver's own
converged pressures every `train_every` steps in the energy norm that CG minimises,
L = (d - e)^T A (d - e) / d^T A d with d = p - p_ext and e = s y(x) (A (d - e) = r_ext - A e, so the
gradient costs one operator apply).  At inference the guess is p_ext + c e + c3 d2, d2 = p^n -
2 p^{n-1} + p^{n-2}, with (c, c3) minimising the residual (two operator applies, a 2x2 system): it
never has a larger residual than p_ext nor than the least-squares third-order extrapolation; when
neither direction reduces the residual the plain extrapolation is used (fallback).  Mode
"extrapolation3" is that third-order baseline without a network.  Feature scaling, the step
lengths and the fallback are computed on the device, so building the guess needs no host round
trip.  All seedings run FP64 CG + FP32 multigrid to the same tolerance, ||r|| <= tol * ||b||.
"""
import time

import exadg_gb300 as E
from exadg_gb300.cnn import CellPatchCNN


def extrapolation_constants(order, time_steps=None, current_order=None):
    """Weights beta_i of p_ext = sum_i beta_i p^{n-i} (ExtrapolationConstants,
    time_integration/extrapolation_constants.cpp:55-150): Lagrange extrapolation through the last
    `current_order` solutions to t_{n+1}, zero-padded to `order` entries (start-up with a lower
    order).  time_steps[j] = t_{n+1-j} - t_{n-j} (time_steps[0] the step being taken); None means
    constant steps.  With nodes tau_0 = 0, tau_i = -(dt_1 + ... + dt_i) relative to t_n and the
    target dt_0: beta_i = prod_{j != i} (dt_0 - tau_j) / (tau_i - tau_j)."""
    q = order if current_order is None else current_order
    if not 1 <= q <= order <= 4:
        raise ValueError("extrapolation order must be 1..4 and current order <= order")
    dt = [1.0] * (q + 1) if time_steps is None else [float(v) for v in time_steps]
    if len(dt) < q:
        raise ValueError("need one time step per extrapolation node")
    tau = [0.0]
    for i in range(1, q):
        tau.append(tau[-1] - dt[i])
    beta = []
    for i in range(q):
        w = 1.0
        for j in range(q):
            if j != i:
                w *= (dt[0] - tau[j]) / (tau[i] - tau[j])
        beta.append(w)
    return beta + [0.0] * (order - q)


def _rms(t):
    import torch

    return float(torch.linalg.norm(t)) / (t.numel() ** 0.5)


class PressureSequence:
    def __init__(self, n_cells=32, degree=2, length=6.283185307179586, mode="learned", train_every=20,
                 epochs=40, lr=1e-4, buffer=20, hidden=32, seed=1, tol=1e-10, outer_precision=E.PREC_F64E,
                 mg_precision=E.PREC_F32, mg_type=E.MG_PH):
        import torch

        self.torch = torch
        kw = dict(n_cells=(n_cells,) * 3, hi=(length,) * 3, periodic=(1, 1, 1))
        self.mesh = E.Mesh(**kw)
        self.op = E.LaplaceOperator(self.mesh, degree, 1.0, outer_precision)
        self.op.tune()
        self.mg = E.MultigridPreconditioner(self.op, mg_precision=mg_precision, singular=True, mg_type=mg_type)
        self.n_cells = n_cells
        self.nc = n_cells ** 3
        self.dpc = (degree + 1) ** 3
        self.mode = mode
        self.train_every = train_every
        self.epochs = epochs
        self.lr = lr
        self.buffer_size = buffer
        self.tol = tol
        self.hist = []  # converged pressures, newest last
        self.samples = []
        self.cnn = None
        if mode in ("learned", "untrained"):
            self.cnn = CellPatchCNN((n_cells,) * 3, 4 * self.dpc, hidden, self.dpc, seed)
            # the linear skip starts as the third-order extrapolation term: output = input channels of
            # the second backward difference p^n - 2 p^{n-1} + p^{n-2}
            off = sum(int(torch.tensor(sh).prod()) for _, sh in self.cnn.layer_shapes()[:6])
            w4 = self.cnn.params[off:off + self.dpc * 4 * self.dpc].view(self.dpc, 4 * self.dpc)
            w4.zero_()
            w4[:, 2 * self.dpc:3 * self.dpc] += torch.eye(self.dpc, device="cuda")
            # the last convolution (W3, b3) starts at zero, so the untrained network is exactly the
            # third-order term and training learns a correction to it
            shapes = self.cnn.layer_shapes()
            o3 = sum(int(torch.tensor(sh).prod()) for _, sh in shapes[:4])
            n3 = sum(int(torch.tensor(sh).prod()) for _, sh in shapes[4:6])
            self.cnn.params[o3:o3 + n3].zero_()
            self.w4_slice = (off, off + self.dpc * 4 * self.dpc)
        self.trained = mode == "untrained"
        self.delta_scale = None
        self.x = torch.empty((4 * self.dpc, self.nc), dtype=torch.float32, device="cuda")
        self.log = []
        self.steps_done = 0
        n = self.op.n_dofs
        self.tmp = torch.empty(n, dtype=torch.float64, device="cuda")
        self.zero = torch.zeros(n, dtype=torch.float64, device="cuda")
        self.e = torch.empty(n, dtype=torch.float64, device="cuda")
        self.Ae = torch.empty(n, dtype=torch.float64, device="cuda")
        self.Af = torch.empty(n, dtype=torch.float64, device="cuda")
        self.rms = torch.empty(4, dtype=torch.float64, device="cuda")
        self.diagnostics = False

    # ------------------------------------------------------------------------------------------
    def _residual(self, b, x):
        return self.op.residual(self.torch.empty_like(x), b, x)

    def _extrapolation(self):
        """BDF2 extrapolation 2 p^n - p^{n-1} (one kernel)."""
        return self.torch.lerp(self.hist[-2], self.hist[-1], 2.0)

    def _features(self, b, p_ext):
        """Network input from (p^n, p^n - p^{n-1}, p^n - 2 p^{n-1} + p^{n-2}, b - A p_ext) on the device;
        each is scaled by its RMS except the second difference, which is scaled by the running RMS
        of the corrections (the scale of the output), so that the linear skip reproduces the
        third-order term exactly.  Returns r_ext = b - A p_ext.  No host round trip."""
        r_ext = self.torch.empty_like(p_ext)
        self.op.residual(r_ext, b, p_ext)
        E._check(E._lib.exg_dg_features(E._ptr(self.hist[-1]), E._ptr(self.hist[-2]), E._ptr(self.hist[-3]),
                                        E._ptr(r_ext), self.dpc, self.nc, self.delta_scale or 0.0, E._ptr(self.x),
                                        E._ptr(self.rms), E._stream()))
        return r_ext

    def _second_difference(self):
        """p^n - 2 p^{n-1} + p^{n-2}: the third-order extrapolation adds it to p_ext."""
        d2 = self.hist[-1] - self.hist[-2]
        d2 -= self.hist[-2]
        d2 += self.hist[-3]
        return d2

    def initial_guess(self, b):
        """Returns (guess, info).  The learned branch runs without a host round trip: the step length
        of the correction and the fallback decision are taken on the device (exg_dg_ls_step); the
        statistics behind them are read after the solve (info["stats"])."""
        torch = self.torch
        info = {"source": "zero"}
        if len(self.hist) == 0:
            return torch.zeros_like(b), info
        if len(self.hist) == 1:
            info["source"] = "previous"
            return self.hist[-1].clone(), info
        p_ext = self._extrapolation()
        info["source"] = "extrapolation"
        x = torch.empty_like(p_ext)
        stats = torch.empty(6, dtype=torch.float64, device="cuda")
        if self.mode == "extrapolation3" and len(self.hist) >= 3:
            # baseline without a network: p_ext + c (p^n - 2 p^{n-1} + p^{n-2}), c by least squares
            r_ext = self._residual(b, p_ext)
            d2 = self._second_difference()
            self.op.vmult(self.Ae, d2)
            E._check(E._lib.exg_dg_ls_step(E._ptr(r_ext), E._ptr(self.Ae), E._ptr(d2), None, None, E._ptr(p_ext),
                                           self.op.n_dofs, E._ptr(x), E._ptr(stats), E._stream()))
            info["stats"] = stats
            info["kind"] = "extrapolation3"
            return x, info
        if self.cnn is None or len(self.hist) < 3 or not self.trained or self.delta_scale is None:
            return p_ext, info
        r_ext = self._features(b, p_ext)
        y = self.cnn.forward(self.x)
        E._check(E._lib.exg_dg_unpack_add(E._ptr(y), E._ptr(self.zero), self.delta_scale, self.dpc, self.nc,
                                          E._ptr(self.e), E._stream()))
        self.op.vmult(self.Ae, self.e)
        # least squares over span{e, p^n - 2 p^{n-1} + p^{n-2}}: never worse than either direction
        d2 = self._second_difference()
        self.op.vmult(self.Af, d2)
        E._check(E._lib.exg_dg_ls_step(E._ptr(r_ext), E._ptr(self.Ae), E._ptr(self.e), E._ptr(self.Af), E._ptr(d2),
                                       E._ptr(p_ext), self.op.n_dofs, E._ptr(x), E._ptr(stats), E._stream()))
        info["stats"] = stats
        info["kind"] = "learned"
        if self.diagnostics:  # residual of the third-order extrapolation p_ext + (p^n - 2p^{n-1} + p^{n-2})
            d2 = self.hist[-1] - 2 * self.hist[-2] + self.hist[-3]
            info["r_ext3"] = float(torch.linalg.norm(self._residual(b, p_ext + d2)))
        return x, info

    @staticmethod
    def _resolve(info):
        """Reads the device statistics of a learned guess (after the solve has synchronised)."""
        if "stats" not in info:
            return info
        rae, aa, rr, ce, cf, red = info.pop("stats").tolist()
        info["c"] = ce
        info["c_d2"] = cf
        info["r_ext"] = rr ** 0.5
        info["r_cnn"] = max(rr - red, 0.0) ** 0.5
        kind = info.pop("kind")
        if kind == "extrapolation3":
            info["source"] = "extrapolation3" if ce != 0.0 else "fallback"
        else:
            info["source"] = "learned" if (ce != 0.0 or cf != 0.0) else "fallback"
        return info

    def _record_sample(self, b, p_new):
        """Training sample: features at the state before the solve and r_ext = b - A p_ext."""
        if self.cnn is None or len(self.hist) < 3:
            return
        p_ext = self._extrapolation()
        delta = p_new - p_ext
        s = _rms(delta)
        self.delta_scale = s if self.delta_scale is None else 0.8 * self.delta_scale + 0.2 * s
        r_ext = self._features(b, p_ext)
        self.samples.append((self.x.clone(), r_ext, delta))
        if len(self.samples) > self.buffer_size:
            self.samples.pop(0)

    def _train(self):
        """Adam steps on L = (d - e)^T A (d - e) / d^T A d with e = s y(x) in DG layout:
        dL/de = -2 (r_ext - A e) / (d . r_ext) (A symmetric, A d = r_ext); dL/dy = s dL/de."""
        torch = self.torch
        s = self.delta_scale
        zero = torch.zeros(self.op.n_dofs, dtype=torch.float64, device="cuda")
        e = torch.empty_like(zero)
        Ae = torch.empty_like(zero)
        gy = torch.empty((self.dpc, self.nc), dtype=torch.float32, device="cuda")
        losses = []
        for it in range(self.epochs):
            x, r_ext, d = self.samples[it % len(self.samples)]
            nrm = float(d @ r_ext)
            y = self.cnn.forward(x)
            E._check(E._lib.exg_dg_unpack_add(E._ptr(y), E._ptr(zero), s, self.dpc, self.nc, E._ptr(e), E._stream()))
            self.op.vmult(Ae, e)
            res = r_ext - Ae
            losses.append(float((d - e) @ res) / nrm)
            # gy[i][c] = s * (-2 / nrm) * res[c*dpc + i]
            E._check(E._lib.exg_dg_pack_diff(E._ptr(zero), E._ptr(res), 2.0 * s / nrm, self.dpc, self.nc,
                                             E._ptr(gy), E._stream()))
            self.cnn.backward(x, gy)
            # the skip stays the third-order term (Adam's sign-like first steps would only perturb
            # it); the convolutions learn the correction to it
            self.cnn.grads[self.w4_slice[0]:self.w4_slice[1]].zero_()
            self.cnn.adam(self.lr)
        self.trained = True
        return losses

    # ------------------------------------------------------------------------------------------
    def step(self, b):
        torch = self.torch
        b = b - b.mean()  # singular periodic problem: project the rhs (operator_projection_methods.cpp)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x, info = self.initial_guess(b)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        bn = float(torch.linalg.norm(b))
        solver = E.KrylovSolver(self.op, self.mg, rel_tol=1e-30, abs_tol=self.tol * bn, max_iter=1000)
        its = solver.solve(x, b)
        x -= x.mean()  # fix the pressure level of the singular problem
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        info = self._resolve(info)
        rec = dict(step=self.steps_done, iterations=its, solve_s=t2 - t1, guess_s=t1 - t0, source=info["source"],
                   r0_rel=solver.result["r0"] / bn)
        if "r_ext" in info:
            rec["r_ext_rel"] = info["r_ext"] / bn
            rec["r_cnn_rel"] = info["r_cnn"] / bn
        if self.mode == "untrained":
            self.samples.clear()
        if "r_ext3" in info:
            rec["r_ext3_rel"] = info["r_ext3"] / bn
        self._record_sample(b, x)
        self.hist.append(x)
        if len(self.hist) > 3:
            self.hist.pop(0)
        if self.mode == "learned" and len(self.samples) > 0 and (self.steps_done + 1) % self.train_every == 0:
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            losses = self._train()
            torch.cuda.synchronize()
            rec["train_s"] = time.perf_counter() - t3
            rec["loss_first"] = losses[0]
            rec["loss_last"] = losses[-1]
        self.log.append(rec)
        self.steps_done += 1
        return x, rec

    # ------------------------------------------------------------------------------------------
    # checkpoint / restart (the state a time loop needs to continue: pressure history, network
    # weights, Adam state, training buffer and scales), as one little-endian file with a header
    _MAGIC = b"EXGPSEQ1"
    _HEADER = "<8sqqqqqqqdq"  # magic, n_dofs, dofs/cell, cells, n_params, n_hist, n_samples, steps,
    #                          delta_scale (NaN: none), flags (bit 0: trained)

    def save(self, path):
        import struct

        import numpy as np

        torch = self.torch
        torch.cuda.synchronize()
        n_params = self.cnn.n_params if self.cnn is not None else 0
        ds = float("nan") if self.delta_scale is None else float(self.delta_scale)
        with open(path, "wb") as f:
            f.write(struct.pack(self._HEADER, self._MAGIC, self.op.n_dofs, self.dpc, self.nc, n_params,
                                len(self.hist), len(self.samples), self.steps_done, ds, int(self.trained)))
            for h in self.hist:
                f.write(h.cpu().numpy().astype("<f8").tobytes())
            if self.cnn is not None:
                m, v, st = self.cnn.optimizer_state()
                for t in (self.cnn.params, m, v):
                    f.write(t.cpu().numpy().astype("<f4").tobytes())
                f.write(np.array([st[0]], dtype="<i8").tobytes())
            for x, r, d in self.samples:
                f.write(x.cpu().numpy().astype("<f4").tobytes())
                f.write(r.cpu().numpy().astype("<f8").tobytes())
                f.write(d.cpu().numpy().astype("<f8").tobytes())

    def load(self, path):
        """Restores a state written by save() into a sequence built with the same mesh, degree
        and mode."""
        import struct

        import numpy as np

        torch = self.torch
        with open(path, "rb") as f:
            head = f.read(struct.calcsize(self._HEADER))
            magic, n, dpc, nc, n_params, n_hist, n_samples, steps, ds, flags = struct.unpack(self._HEADER, head)
            if magic != self._MAGIC:
                raise ValueError("not a pressure-sequence checkpoint")
            own_params = self.cnn.n_params if self.cnn is not None else 0
            if (n, dpc, nc, n_params) != (self.op.n_dofs, self.dpc, self.nc, own_params):
                raise ValueError("checkpoint was written for another mesh, degree or network")

            def read(count, dtype):
                a = np.frombuffer(f.read(count * np.dtype(dtype).itemsize), dtype=dtype)
                if a.size != count:
                    raise ValueError("truncated checkpoint")
                return torch.from_numpy(a.astype(dtype[1:] if dtype[0] == "<" else dtype)).cuda()

            self.hist = [read(n, "<f8") for _ in range(n_hist)]
            if self.cnn is not None:
                m, v, st = self.cnn.optimizer_state()
                self.cnn.params.copy_(read(n_params, "<f4"))
                m.copy_(read(n_params, "<f4"))
                v.copy_(read(n_params, "<f4"))
                st[0] = int(np.frombuffer(f.read(8), dtype="<i8")[0])
            self.samples = []
            for _ in range(n_samples):
                self.samples.append((read(4 * dpc * nc, "<f4").view(4 * dpc, nc), read(n, "<f8"), read(n, "<f8")))
        self.steps_done = steps
        self.delta_scale = None if ds != ds else ds
        self.trained = bool(flags & 1)
        torch.cuda.synchronize()



def tgv_rhs_sequence(n_steps, n_cells=32, degree=2, dt=None, modes=64, device="cuda"):
    """Right-hand sides b^n = (f^n, v) of the DG pressure-Poisson problem along a TGV run."""
    import math

    import torch

    from exadg_gb300.tgv import TGVSpectral, dg_quadrature_grid, grid_to_cells

    if dt is None:  # CFL 0.3 with the velocity degree 3 on n_cells: dt = 0.3 h / (u_max k_u^1.5)
        dt = 0.3 * (2 * math.pi / n_cells) / (3 ** 1.5)
    flow = TGVSpectral(modes=modes, dt=dt, device=device)
    mesh = E.Mesh((n_cells,) * 3, hi=(2 * math.pi,) * 3, periodic=(1, 1, 1))
    op = E.LaplaceOperator(mesh, degree, 1.0, E.PREC_F64)
    xs = dg_quadrature_grid(n_cells, degree + 1, device=device)
    out = []
    for _ in range(n_steps):
        flow.step()
        F = flow.evaluate(flow.pressure_source_hat(), [xs, xs, xs])
        f = grid_to_cells(F, n_cells, degree + 1)
        out.append(op.rhs(f_cell=f))
    return out, dt
