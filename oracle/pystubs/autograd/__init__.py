"""Complex-step stand-in for autograd.grad (test infrastructure only)."""
import numpy as _np


def grad(fun):
    def g(x):
        x = _np.asarray(x, dtype=float)
        h = 1e-30
        out = _np.zeros_like(x)
        for i in range(x.size):
            xc = x.astype(complex)
            xc.flat[i] += 1j * h
            out.flat[i] = _np.imag(fun(xc)) / h
        return out

    return g
