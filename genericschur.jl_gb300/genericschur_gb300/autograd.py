"""torch.autograd.Function for batched complex eigenvalues (the Python analogue of
a ChainRulesCore rrule): forward = batched Schur on the GPU, keeping only T and Z;
backward = eigenvectors recomputed from (T, Z) and the eigenvalue adjoint
grad = sum_i gbar_i y_i x_i^H / conj(y_i^H x_i), both in the CUDA library.

Tensors are complex128 of shape (batch, n, n) on a CUDA device; the library is
driven through its device-pointer entry points on the current torch stream.
"""
import torch

from . import _capi
from ._capi import GS_DEVICE, GS_SCALE, GS_WANTZ, get_context


def _meta(batch, n, device):
    ns = torch.full((batch,), n, dtype=torch.int32, device=device)
    offs = torch.arange(batch, dtype=torch.int64, device=device) * (n * n)
    woffs = torch.arange(batch, dtype=torch.int64, device=device) * n
    return ns, offs, woffs


class BatchedEigvals(torch.autograd.Function):
    @staticmethod
    def forward(ctx_, A):
        assert A.is_cuda and A.dtype == torch.complex128 and A.dim() == 3 and A.shape[1] == A.shape[2]
        batch, n, _ = A.shape
        lib_ctx = get_context(A.device.index or 0)
        lib_ctx.set_stream(torch.cuda.current_stream(A.device).cuda_stream or 1)
        # column-major per matrix: transpose the trailing dims into a contiguous buffer
        T = A.transpose(1, 2).contiguous()
        Z = torch.empty_like(T)
        w = torch.empty(batch * n, dtype=torch.complex128, device=A.device)
        st = torch.empty(batch, dtype=torch.int32, device=A.device)
        ns, offs, woffs = _meta(batch, n, A.device)
        rc = lib_ctx.lib.gs_schur_batched_c64(lib_ctx.handle, batch, ns.data_ptr(), offs.data_ptr(), woffs.data_ptr(),
                                              T.data_ptr(), Z.data_ptr(), w.data_ptr(), st.data_ptr(),
                                              GS_WANTZ | GS_SCALE | GS_DEVICE)
        if rc != 0:
            raise RuntimeError("gs_schur_batched_c64: %s" % lib_ctx.last_error())
        # per-matrix status: a matrix that hit the iteration limit has no Schur form to
        # differentiate, and the reference raises UnconvergedException for it
        # (GenericSchur.jl:39-45, 553-556); an order the kernel rejected is an ArgumentError
        bad = torch.nonzero(st != 0).flatten().cpu()
        if bad.numel():
            from . import ArgumentError, UnconvergedException
            b0 = int(bad[0])
            code = int(st[b0].item())
            msg = "matrix %d of the batch (%d failed): status %d" % (b0, bad.numel(), code)
            if code == _capi.GS_UNCONVERGED:
                raise UnconvergedException("Convergence failure; " + msg)
            raise ArgumentError(msg)
        ctx_.save_for_backward(T, Z, ns, offs, woffs)
        return w.view(batch, n)

    @staticmethod
    def backward(ctx_, gw):
        T, Z, ns, offs, woffs = ctx_.saved_tensors
        batch = ns.shape[0]
        n = T.shape[1]
        lib_ctx = get_context(T.device.index or 0)
        lib_ctx.set_stream(torch.cuda.current_stream(T.device).cuda_stream or 1)
        g = gw.contiguous().view(-1).to(torch.complex128)
        G = torch.empty_like(T)
        rc = lib_ctx.lib.gs_eig_adjoint_batched_c64(lib_ctx.handle, batch, ns.data_ptr(), offs.data_ptr(),
                                                    woffs.data_ptr(), batch * n * n, batch * n, T.data_ptr(),
                                                    Z.data_ptr(), g.data_ptr(), G.data_ptr(), GS_DEVICE)
        if rc != 0:
            raise RuntimeError("gs_eig_adjoint_batched_c64: %s" % lib_ctx.last_error())
        return G.transpose(1, 2)


def eigvals_batched(A):
    """Differentiable eigenvalues of a (batch, n, n) complex128 CUDA tensor."""
    return BatchedEigvals.apply(A)
