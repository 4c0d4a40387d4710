"""Gradient form over the C ABI's iris_adjoint_* entry points.

The objective is L = sum_w w5[w] J5(w) + w6[w] J6(w), the weighted reflection
and transmission fluxes of box 1 (scattering_fourier_out,
code/dataprocess.f90:246-277), as a function of the permittivity of a design
region inside the structure layer (eps_inv of slit()/set_emconstants,
code/mesh.f90:57-109).  The gradient comes from the engine's hand-written
time-reversed adjoint kernels, with checkpoints every ``checkpoint_every``
steps and recomputation of each segment during the backward sweep.

``design_objective`` wraps one ``Adjoint`` in a ``torch.autograd.Function``:
eps (the design region's relative permittivity, real) -> L, whose backward
is dL/d eps = -eps_inv**2 dL/d eps_inv.  PyTorch is only the wrapper: both
solves run in the CUDA engine on host copies of the tensors.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .native import IrisParams, check, lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Adjoint:
    """iris_adjoint: forward solve with checkpoints, then dL/d eps_inv.

    design = (x0, x1, y0, y1, z0, z1), 1-based inclusive, inside
    [1,nx] x [1,ny] x [hi,hf]; weights = (w5, w6) arrays of nof or None (J6)."""

    def __init__(self, params: IrisParams, fw, design, checkpoint_every: int = 256, weights=None,
                 precision: int | None = None, device: int = 0):
        self.L = lib()
        q = params.copy()
        if precision is not None:
            q.precision = precision
        q.device = device
        q.dft_block = 0
        self.p = q
        self.fw = np.ascontiguousarray(np.asarray(fw, dtype=np.float64))
        self.design = tuple(int(v) for v in design)
        x0, x1, y0, y1, z0, z1 = self.design
        self.shape = (z1 - z0 + 1, y1 - y0 + 1, x1 - x0 + 1)
        d = (ctypes.c_int * 6)(*self.design)
        w = None
        if weights is not None:
            w = np.ascontiguousarray(np.concatenate([np.asarray(weights[0], float), np.asarray(weights[1], float)]))
            if w.size != 2 * q.nof:
                raise ValueError("weights must be two arrays of nof values")
        self._w = w
        h = ctypes.c_void_p()
        check(self.L.iris_adjoint_create(ctypes.byref(q), _dp(self.fw), d, int(checkpoint_every),
                                         _dp(w) if w is not None else None, ctypes.byref(h)), "iris_adjoint_create")
        self.h = h
        self.nsteps = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.iris_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_material(self, eps_inv: np.ndarray):
        from . import _split_material

        p = self.p
        want = (p.hf - p.hi + 3, p.ny + 2, p.nx + 2)
        if np.shape(eps_inv) != want:
            raise ValueError(f"eps_inv shape {np.shape(eps_inv)} != {want}")
        re, im = _split_material(eps_inv)
        check(self.L.iris_adjoint_set_material(self.h, _dp(re), _dp(im) if im is not None else None),
              "iris_adjoint_set_material")

    def set_design(self, eps_inv: np.ndarray):
        """eps_inv of the design cells, shape (nz, ny, nx) of the region."""
        a = np.ascontiguousarray(np.asarray(eps_inv, dtype=np.float64))
        if a.shape != self.shape:
            raise ValueError(f"design shape {a.shape} != {self.shape}")
        check(self.L.iris_adjoint_set_design(self.h, _dp(a)), "iris_adjoint_set_design")

    def forward(self, nsteps: int):
        """Steps 1..nsteps from zero fields: (L, J[6, nof])."""
        Lv = ctypes.c_double(0)
        J = np.zeros(6 * self.p.nof)
        check(self.L.iris_adjoint_forward(self.h, int(nsteps), ctypes.byref(Lv), _dp(J)), "iris_adjoint_forward")
        self.nsteps = nsteps
        return Lv.value, J.reshape(6, -1)

    def backward(self) -> np.ndarray:
        """dL/d eps_inv over the design cells, shape (nz, ny, nx)."""
        g = np.zeros(self.shape)
        check(self.L.iris_adjoint_backward(self.h, _dp(g)), "iris_adjoint_backward")
        return g

    def engine(self, which: int):
        """Borrowed view of the forward engine (0) or of the adjoint state (1)."""
        from . import Engine

        e = ctypes.c_void_p()
        check(self.L.iris_adjoint_engine(self.h, which, ctypes.byref(e)), "iris_adjoint_engine")
        return Engine._view(e, self.p, self.fw, self)

    def apply(self, nsteps: int = 1):
        check(self.L.iris_adjoint_apply(self.h, int(nsteps)), "iris_adjoint_apply")

    def timing(self) -> dict:
        ms = np.zeros(3)
        check(self.L.iris_adjoint_timing(self.h, _dp(ms)), "iris_adjoint_timing")
        return dict(forward_ms=ms[0], recompute_ms=ms[1], adjoint_ms=ms[2])


def design_objective(adj: Adjoint, nsteps: int):
    """A function eps -> L (torch tensors) whose backward runs the adjoint.

    eps: real tensor of the design region's shape (nz, ny, nx) holding the
    relative permittivity; the result is a 0-d float64 tensor on eps.device."""
    import torch

    class _Objective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, eps):
            e = eps.detach().to("cpu", torch.float64).numpy()
            adj.set_design(1.0 / e)
            L, _ = adj.forward(nsteps)
            ctx.save_for_backward(eps)
            return torch.tensor(L, dtype=torch.float64, device=eps.device)

        @staticmethod
        def backward(ctx, gL):
            (eps,) = ctx.saved_tensors
            g = adj.backward()
            e = eps.detach().to("cpu", torch.float64).numpy()
            dL = -g / (e * e)
            return gL * torch.from_numpy(dL).to(device=eps.device, dtype=eps.dtype)

    return _Objective.apply
