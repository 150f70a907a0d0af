"""Pressure-Poisson right-hand sides of the Taylor-Green vortex (Re = 1600) on [0, 2 pi]^3.

The reference produces this sequence with its incompressible dual-splitting solver
(TimeIntBDFDualSplitting::pressure_step, time_int_bdf_dual_splitting.cpp:480-530;
applications/incompressible_navier_stokes/taylor_green_vortex/application.h).  That solver is not
part of this library's scope, so a pseudo-spectral Navier-Stokes integrator (rotational form, 2/3
de-aliasing, classical RK4; torch FFTs) advances the same flow, and at every step the pressure
source of the incompressible equations, -Laplace p = d_i d_j (u_i u_j), is evaluated at the DG
quadrature points.  The DG pressure-Poisson problem (SIPG, k_p, periodic, singular) solved on it is
the reference's PPE with a right-hand side from an exactly divergence-free velocity.
"""
import math


class TGVSpectral:
    def __init__(self, modes=64, nu=1.0 / 1600.0, dt=0.01, device="cuda"):
        import torch

        self.torch = torch
        self.M = modes
        self.nu = nu
        self.dt = dt
        self.t = 0.0
        M = modes
        k1 = torch.fft.fftfreq(M, d=1.0 / M).to(device=device, dtype=torch.float64)
        kz, ky, kx = torch.meshgrid(k1, k1, k1, indexing="ij")  # arrays indexed [z, y, x]
        self.k = [kx, ky, kz]
        self.k2 = kx * kx + ky * ky + kz * kz
        self.k2inv = torch.where(self.k2 > 0, 1.0 / self.k2, torch.zeros_like(self.k2))
        kmax = M // 3
        self.dealias = ((kx.abs() <= kmax) & (ky.abs() <= kmax) & (kz.abs() <= kmax)).to(torch.float64)
        x1 = torch.arange(M, device=device, dtype=torch.float64) * (2 * math.pi / M)
        z, y, x = torch.meshgrid(x1, x1, x1, indexing="ij")
        u = torch.sin(x) * torch.cos(y) * torch.cos(z)
        v = -torch.cos(x) * torch.sin(y) * torch.cos(z)
        w = torch.zeros_like(u)
        self.uh = [torch.fft.fftn(c) for c in (u, v, w)]

    def _rhs(self, uh):
        torch = self.torch
        k = self.k
        u = [torch.fft.ifftn(c).real for c in uh]
        # vorticity
        wx = torch.fft.ifftn(1j * (k[1] * uh[2] - k[2] * uh[1])).real
        wy = torch.fft.ifftn(1j * (k[2] * uh[0] - k[0] * uh[2])).real
        wz = torch.fft.ifftn(1j * (k[0] * uh[1] - k[1] * uh[0])).real
        n = [u[1] * wz - u[2] * wy, u[2] * wx - u[0] * wz, u[0] * wy - u[1] * wx]  # u x omega
        nh = [torch.fft.fftn(c) * self.dealias for c in n]
        kdot = (k[0] * nh[0] + k[1] * nh[1] + k[2] * nh[2]) * self.k2inv
        return [nh[i] - k[i] * kdot - self.nu * self.k2 * uh[i] for i in range(3)]

    def step(self):
        dt = self.dt
        u0 = self.uh
        a = self._rhs(u0)
        b = self._rhs([u0[i] + 0.5 * dt * a[i] for i in range(3)])
        c = self._rhs([u0[i] + 0.5 * dt * b[i] for i in range(3)])
        d = self._rhs([u0[i] + dt * c[i] for i in range(3)])
        self.uh = [u0[i] + dt / 6.0 * (a[i] + 2 * b[i] + 2 * c[i] + d[i]) for i in range(3)]
        self.t += dt

    def pressure_source_hat(self):
        """Fourier coefficients of d_i d_j (u_i u_j) (= -Laplace p), de-aliased."""
        torch = self.torch
        u = [torch.fft.ifftn(c).real for c in self.uh]
        f = torch.zeros_like(self.uh[0])
        for i in range(3):
            for j in range(i, 3):
                h = torch.fft.fftn(u[i] * u[j]) * self.dealias
                term = -self.k[i] * self.k[j] * h
                f = f + (term if i == j else 2 * term)
        return f

    def evaluate(self, fh, xs):
        """Values of the real field with coefficients fh at the tensor grid xs[0] x xs[1] x xs[2]
        (1D coordinate tensors); returns an array indexed [z, y, x]."""
        torch = self.torch
        M = self.M
        k1 = torch.fft.fftfreq(M, d=1.0 / M).to(device=fh.device, dtype=torch.float64)
        E = [torch.exp(1j * torch.outer(x, k1)) for x in xs]  # [P_d, M]
        t = torch.einsum("zyx,ax->zya", fh, E[0])
        t = torch.einsum("zya,by->zba", t, E[1])
        t = torch.einsum("zba,cz->cba", t, E[2])
        return t.real / (M ** 3)


def dg_quadrature_grid(n_cells, nq, length=2 * math.pi, device="cuda"):
    """1D coordinates of the Gauss points of all cells (cell-major, point-minor)."""
    import numpy as np
    import torch

    x, _ = np.polynomial.legendre.leggauss(nq)
    g = 0.5 * (x + 1.0)
    h = length / n_cells
    pts = np.array([(c + gq) * h for c in range(n_cells) for gq in g])
    return torch.tensor(pts, dtype=torch.float64, device=device)


def grid_to_cells(F, n_cells, nq):
    """[z][y][x] values on the tensor grid -> [cell][q] in the library's layout (cells x-fastest,
    points x-fastest)."""
    n = n_cells
    G = F.reshape(n, nq, n, nq, n, nq)  # cz, q2, cy, q1, cx, q0
    G = G.permute(0, 2, 4, 1, 3, 5)  # cz, cy, cx, q2, q1, q0
    return G.reshape(n * n * n * nq ** 3).contiguous()
