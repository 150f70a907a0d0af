"""NumPy restatement of the cell-patch CNN (forward and backward) -- TEST INFRASTRUCTURE ONLY.

Checks the hand-written CUDA kernels of exadg_gb300/csrc/cnn.cu: the same network (1x1x1, two
3x3x3 periodic convolutions, SiLU), the same parameter layout (W1 [hid][in], b1, W2 [hid][hid][27],
b2, W3 [out][hid][27], b3, W4 [out][in] -- the linear skip) and channel-major activations [C][n_cells] with cells x-fastest.
Computed in float64."""
import numpy as np


def split(params, c_in, c_hid, c_out):
    o = 0
    out = []
    for shape in [(c_hid, c_in), (c_hid,), (c_hid, c_hid, 27), (c_hid,), (c_out, c_hid, 27), (c_out,), (c_out, c_in)]:
        n = int(np.prod(shape))
        out.append(np.asarray(params[o:o + n], dtype=np.float64).reshape(shape))
        o += n
    return out


def shift(a, N, t):
    """a[C][cells] -> a[:, nb(c, t)] with periodic wrap (tap t = dx + 3 dy + 9 dz, d in {-1,0,1})."""
    dx, dy, dz = t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1
    C = a.shape[0]
    g = a.reshape(C, N[2], N[1], N[0])
    g = np.roll(g, shift=(-dz, -dy, -dx), axis=(1, 2, 3))
    return g.reshape(C, -1)


def conv3(W, b, a, N):
    y = np.zeros((W.shape[0], a.shape[1]))
    for t in range(27):
        y += W[:, :, t] @ shift(a, N, t)
    if b is not None:
        y += b[:, None]
    return y


def silu(v):
    return v / (1.0 + np.exp(-v))


def silu_grad(v):
    s = 1.0 / (1.0 + np.exp(-v))
    return s * (1.0 + v * (1.0 - s))


def forward(params, x, N, c_in, c_hid, c_out):
    W1, b1, W2, b2, W3, b3, W4 = split(params, c_in, c_hid, c_out)
    p1 = W1 @ x + b1[:, None]
    a1 = silu(p1)
    p2 = conv3(W2, b2, a1, N)
    a2 = silu(p2)
    y = conv3(W3, b3, a2, N) + W4 @ x
    return y, (p1, a1, p2, a2)


def backward(params, x, gy, N, c_in, c_hid, c_out):
    """Gradient of <gy, y(x)> with respect to the parameter vector."""
    W1, b1, W2, b2, W3, b3, W4 = split(params, c_in, c_hid, c_out)
    y, (p1, a1, p2, a2) = forward(params, x, N, c_in, c_hid, c_out)
    gW4 = gy @ x.T
    gW3 = np.stack([gy @ shift(a2, N, t).T for t in range(27)], axis=2)
    gb3 = gy.sum(axis=1)
    ga2 = np.zeros_like(a2)
    for t in range(27):
        # adjoint of the shift: roll back
        ga2 += shift(W3[:, :, t].T @ gy, N, 26 - t)
    g2 = ga2 * silu_grad(p2)
    gW2 = np.stack([g2 @ shift(a1, N, t).T for t in range(27)], axis=2)
    gb2 = g2.sum(axis=1)
    ga1 = np.zeros_like(a1)
    for t in range(27):
        ga1 += shift(W2[:, :, t].T @ g2, N, 26 - t)
    g1 = ga1 * silu_grad(p1)
    gW1 = g1 @ x.T
    gb1 = g1.sum(axis=1)
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3, gW4.ravel()])
