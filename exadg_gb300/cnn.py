"""Python handle of the cell-patch CNN (csrc/cnn.cu) used for the learned initial guess."""
import ctypes

import exadg_gb300 as E


class _CudaArray:
    """Minimal __cuda_array_interface__ wrapper to view library-owned device memory in torch."""

    def __init__(self, ptr, n, typestr="<f4"):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                         "strides": None}


class CellPatchCNN:
    """1x1x1 c_in->c_hid, 3x3x3 c_hid->c_hid, 3x3x3 c_hid->c_out with SiLU, periodic padding, plus a
    linear 1x1x1 skip c_in->c_out."""

    def __init__(self, n_cells, c_in=108, c_hidden=32, c_out=27, seed=1):
        L = E.load_library()
        n = (ctypes.c_int * 3)(*n_cells)
        h = ctypes.c_void_p()
        E._check(L.exg_cnn_create(n, c_in, c_hidden, c_out, seed, ctypes.byref(h)))
        self.h = h
        self.n_cells = tuple(n_cells)
        self.c_in, self.c_hidden, self.c_out = c_in, c_hidden, c_out
        cnt = ctypes.c_longlong()
        E._check(L.exg_cnn_n_params(h, ctypes.byref(cnt)))
        self.n_params = cnt.value

    def __del__(self):
        if getattr(self, "h", None) and E._lib is not None:
            E._lib.exg_cnn_destroy(self.h)
            self.h = None

    def _views(self):
        import torch

        p = ctypes.c_void_p()
        g = ctypes.c_void_p()
        E._check(E._lib.exg_cnn_params(self.h, ctypes.byref(p), ctypes.byref(g)))
        return (torch.as_tensor(_CudaArray(p.value, self.n_params), device="cuda"),
                torch.as_tensor(_CudaArray(g.value, self.n_params), device="cuda"))

    @property
    def params(self):
        """Device view of the parameter vector (W1, b1, W2, b2, W3, b3, W4)."""
        return self._views()[0]

    @property
    def grads(self):
        return self._views()[1]

    def optimizer_state(self):
        """(first moments, second moments) as device views, and the Adam step count."""
        import torch

        m = ctypes.c_void_p()
        v = ctypes.c_void_p()
        st = ctypes.POINTER(ctypes.c_longlong)()
        E._check(E._lib.exg_cnn_optimizer_state(self.h, ctypes.byref(m), ctypes.byref(v), ctypes.byref(st)))
        return (torch.as_tensor(_CudaArray(m.value, self.n_params), device="cuda"),
                torch.as_tensor(_CudaArray(v.value, self.n_params), device="cuda"), st)

    @property
    def adam_step(self):
        return self.optimizer_state()[2][0]

    @adam_step.setter
    def adam_step(self, value):
        self.optimizer_state()[2][0] = int(value)

    def layer_shapes(self):
        ci, ch, co = self.c_in, self.c_hidden, self.c_out
        return [("W1", (ch, ci)), ("b1", (ch,)), ("W2", (ch, ch, 27)), ("b2", (ch,)), ("W3", (co, ch, 27)),
                ("b3", (co,)), ("W4", (co, ci))]

    def forward(self, x, y=None, stream=None):
        import torch

        nc = self.n_cells[0] * self.n_cells[1] * self.n_cells[2]
        if y is None:
            y = torch.empty((self.c_out, nc), dtype=torch.float32, device="cuda")
        E._check(E._lib.exg_cnn_forward(self.h, E._ptr(x), E._ptr(y), E._stream(stream)))
        return y

    def backward(self, x, gy, stream=None):
        E._check(E._lib.exg_cnn_backward(self.h, E._ptr(x), E._ptr(gy), E._stream(stream)))
        return self.grads

    def adam(self, lr=1e-3, stream=None):
        """Adam update with the gradient left by backward()."""
        E._check(E._lib.exg_cnn_adam(self.h, lr, E._stream(stream)))

    def train_step(self, x, target, lr=1e-3, stream=None):
        loss = ctypes.c_float()
        E._check(E._lib.exg_cnn_train_step(self.h, E._ptr(x), E._ptr(target), lr, ctypes.byref(loss),
                                           E._stream(stream)))
        return loss.value
