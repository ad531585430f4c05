"""Reconstruction quality over the C ABI (pvvc_cloud_quality): the
symmetric nearest-neighbour geometry and Y/U/V errors of two coloured clouds
-- common::MSE::Compute (src/registration/registration_base.cc:160-223) --
and the decoder's PSNR (src/codec/pvvc_decompression.cc:151-171).

Device buffers are torch tensors (plumbing only); the work runs in
libpvvc_gb300.so."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L


def _dev(torch, a, dtype, dev):
    if isinstance(a, torch.Tensor):
        return a.to(dev, dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype)


class Quality:
    """Grows its workspace as needed; one call per pair of clouds."""

    def __init__(self, device="cuda"):
        import torch
        self.torch = torch
        self.dev = torch.device(device)
        self.ws = torch.empty(256, dtype=torch.uint8, device=self.dev)
        self.out = torch.zeros(8, dtype=torch.float64, device=self.dev)

    def mse(self, a_xyz, a_rgb, b_xyz, b_rgb, stream=None) -> np.ndarray:
        """[geo A->B, geo B->A, Y A->B, Y B->A, U.., U.., V.., V..] (A is the
        reference's p_, B its q_).  Inputs: numpy arrays or device tensors."""
        torch = self.torch
        ax = _dev(torch, a_xyz, torch.float32, self.dev).reshape(-1, 3)
        ac = _dev(torch, a_rgb, torch.uint8, self.dev).reshape(-1, 3)
        bx = _dev(torch, b_xyz, torch.float32, self.dev).reshape(-1, 3)
        bc = _dev(torch, b_rgb, torch.uint8, self.dev).reshape(-1, 3)
        na, nb = ax.shape[0], bx.shape[0]
        need = C.c_uint64(0)
        L.check(L.lib().pvvc_cloud_quality_workspace_size(na, nb, C.byref(need)), "pvvc_cloud_quality_workspace_size")
        if self.ws.numel() < need.value:
            self.ws = torch.empty(int(need.value), dtype=torch.uint8, device=self.dev)
        sp = stream if stream is not None else torch.cuda.current_stream(self.dev).cuda_stream
        L.check(L.lib().pvvc_cloud_quality(na, ax.data_ptr(), ac.data_ptr(), nb, bx.data_ptr(), bc.data_ptr(),
                                           self.out.data_ptr(), self.ws.data_ptr(), self.ws.numel(), sp),
                "pvvc_cloud_quality")
        return self.out.cpu().numpy().copy()


def psnr(mse8: np.ndarray, peak_geo: float = 1024.0, peak_color: float = 256.0) -> dict:
    """PSNR as PVVCDecompression reports it (pvvc_decompression.cc:157-160):
    the larger of the two directions, 10 log10(peak^2 / mse); infinite for a
    zero error."""
    def p(m, peak):
        return math.inf if m <= 0 else 10.0 * math.log10(peak * peak / m)
    g, y, u, v = (max(mse8[2 * k], mse8[2 * k + 1]) for k in range(4))
    return {"geo": p(g, peak_geo), "y": p(y, peak_color), "u": p(u, peak_color), "v": p(v, peak_color),
            "mse_geo": g, "mse_y": y, "mse_u": u, "mse_v": v}
