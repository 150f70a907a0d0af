"""GPU-test helpers: build/load the library, paired oracle / device problems."""
import numpy as np
import pytest

import exadg_gb300 as E
import oracle as O
from tests.helpers import mesh_kwargs, splitmix_uniform


def require_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from exadg_gb300 import build as B

    B.build()
    E.load_library()
    return torch


def pair(kind, n, k, prec=E.PREC_F64):
    kw = mesh_kwargs(kind, n)
    p = O.Problem(O.mesh_desc(**kw), k)
    m = E.Mesh(**kw)
    op = E.LaplaceOperator(m, k, 1.0, prec)
    return p, m, op


def to_dev(torch, x, dtype=None):
    return torch.tensor(np.asarray(x), dtype=dtype or torch.float64, device="cuda")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)
