"""Differentiable Dij: dose = D.w as a torch.autograd.Function over the C ABI.

The Dij scorer (moqui's DOSE_Dij, scored into insert_hashtable's (voxel, spot) table,
moqui/kernel_functions/mqi_transport.hpp:68-111, and written as a spot-row CSR by save_to_npz,
moqui/base/mqi_io.hpp:251-320) is built on the device into two CSR layouts by mqi_dij_build.  The
forward product gathers over voxel rows; the backward product D^T.g gathers over spot rows (the
transposed layout, which is also the reference's npz layout).  Both run on torch's current CUDA
stream through device pointers; PyTorch only provides the tensors and the autograd graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi


class DijOperator:
    """A built Dij matrix of a context: D has shape [n_voxels, n_spots] (dose = D.w)."""

    def __init__(self, ctx: "capi.Context", scorer_id: int, n_spots: int, n_voxels: int, nnz: int):
        self.ctx = ctx
        self.sid = scorer_id
        self.n_spots = n_spots
        self.n_voxels = n_voxels
        self.nnz = nnz

    def _bind_stream(self, torch):
        # torch's default stream has the handle 0, which the C ABI reads as "the context's own
        # stream"; name the legacy default stream (cudaStreamLegacy = 1) instead so that the
        # products are ordered with the surrounding torch work.
        handle = torch.cuda.current_stream().cuda_stream or 1
        if getattr(self.ctx, "_stream_handle", None) != handle:
            self.ctx.set_stream(handle)
            self.ctx._stream_handle = handle

    def matvec(self, w):
        """dose = D.w for a CUDA tensor w of n_spots entries (float32 or float64)."""
        import torch

        w = w.contiguous()
        if w.numel() != self.n_spots or not w.is_cuda:
            raise ValueError("w must be a CUDA tensor of n_spots entries")
        fp64 = w.dtype == torch.float64
        if not fp64 and w.dtype != torch.float32:
            raise TypeError("w must be float32 or float64")
        out = torch.empty(self.n_voxels, dtype=w.dtype, device=w.device)
        self._bind_stream(torch)
        self.ctx._check(self.ctx.lib.mqi_dij_matvec(self.ctx.h, self.sid, C.c_void_p(w.data_ptr()),
                                                    C.c_void_p(out.data_ptr()), int(fp64), 1), self.ctx.h)
        return out

    def rmatvec(self, g):
        """grad = D^T.g for a CUDA tensor g of n_voxels entries."""
        import torch

        g = g.contiguous()
        if g.numel() != self.n_voxels or not g.is_cuda:
            raise ValueError("g must be a CUDA tensor of n_voxels entries")
        fp64 = g.dtype == torch.float64
        if not fp64 and g.dtype != torch.float32:
            raise TypeError("g must be float32 or float64")
        out = torch.empty(self.n_spots, dtype=g.dtype, device=g.device)
        self._bind_stream(torch)
        self.ctx._check(self.ctx.lib.mqi_dij_rmatvec(self.ctx.h, self.sid, C.c_void_p(g.data_ptr()),
                                                     C.c_void_p(out.data_ptr()), int(fp64), 1), self.ctx.h)
        return out

    def csr(self):
        """Spot-row CSR on the host, the reference's npz layout: (indptr int64 [n_spots+1],
        indices uint32 voxel, data float32), shape (n_spots, n_voxels)."""
        indptr = np.empty(self.n_spots + 1, np.uint64)
        indices = np.empty(self.nnz, np.uint32)
        data = np.empty(self.nnz, np.float32)
        self.ctx._check(self.ctx.lib.mqi_dij_get_csr(self.ctx.h, self.sid, capi._ptr(indptr), capi._ptr(indices),
                                                     capi._ptr(data), 0), self.ctx.h)
        return indptr.astype(np.int64), indices, data

    def save_npz(self, path: str) -> None:
        """Write the spot-row CSR as the reference's save_to_npz does (write_dij_npz)."""
        indptr, indices, data = self.csr()
        write_dij_npz(path, indptr, indices, data, self.n_spots, self.n_voxels)


def write_dij_npz(path: str, indptr, indices, data, n_spots: int, n_voxels: int) -> None:
    """A spot-row CSR in the reference's npz layout (save_to_npz, moqui/base/mqi_io.hpp:251-320,
    with mqi::io::save_npz's dtypes, moqui/base/mqi_sparse_io.hpp:283-330): members indices,
    indptr, shape, data and format, stored uncompressed, with indices, indptr and shape as <u4
    (shape = [n_spots, n_voxels]), data as <f8 and format as |S3 "csr" -- the keys and types
    scipy.sparse.load_npz reads.  The reference's uint32 row pointers cap nnz below 2**32; a
    larger matrix raises rather than wrapping."""
    indptr = np.asarray(indptr)
    if indptr.size != n_spots + 1 or (indptr.size and int(indptr[-1]) != len(indices)):
        raise ValueError("indptr must hold n_spots + 1 row offsets ending at nnz")
    if len(indices) >= 2 ** 32 or n_voxels >= 2 ** 32 or n_spots >= 2 ** 32:
        raise ValueError("the reference's npz layout holds uint32 indices and row offsets")
    np.savez(path, indices=np.asarray(indices, np.uint32), indptr=indptr.astype(np.uint32),
             shape=np.array([n_spots, n_voxels], np.uint32), data=np.asarray(data, np.float64),
             format=np.array(b"csr"))


def _function():
    import torch

    class DijDose(torch.autograd.Function):
        """dose = D.w; backward: grad_w = D^T.grad_dose (hand-written transposed-CSR kernel)."""

        @staticmethod
        def forward(ctx, w, op):
            ctx.op = op
            return op.matvec(w)

        @staticmethod
        def backward(ctx, grad_dose):
            return ctx.op.rmatvec(grad_dose), None

    return DijDose


_DIJ_DOSE = None


def dose(op: DijOperator, w):
    """Differentiable dose = D.w."""
    global _DIJ_DOSE
    if _DIJ_DOSE is None:
        _DIJ_DOSE = _function()
    return _DIJ_DOSE.apply(w, op)
