"""pvvc_icp_batch_noalloc: the registration entry point for callers that cannot
allocate device memory (a host application that owns the GPU's memory, a
per-frame callback that must not synchronise the device).  It must give the
results of pvvc_icp_batch -- within the ICP tests' tolerance -- on two calls
in a row, and refuse batches beyond its fixed scratch.  Collected last on
purpose so that a run stopping at the first failure has run everything else."""
import ctypes as C

import numpy as np
import pytest

ROT_TOL_DEG = 0.1
TRANS_TOL_VOX = 0.1
MSE_RTOL = 0.02

pytestmark = pytest.mark.gpu


def _call_noalloc(pvvc_lib, b, prm, T, mse, iters, conv, npairs=None):
    lib = pvvc_lib.lib()
    return lib.pvvc_icp_batch_noalloc(b.n if npairs is None else npairs, b.src.data_ptr(), b.soff.data_ptr(),
                                      b.tgt.data_ptr(), b.toff.data_ptr(), None, C.byref(prm), T.data_ptr(),
                                      mse.data_ptr(), iters.data_ptr(), conv.data_ptr(), b.nt,
                                      b.torch.cuda.current_stream().cuda_stream)


def test_icp_noalloc_matches_workspace_entry(pvvc_lib):
    import torch
    assert torch.cuda.is_available()
    from pvvc import _lib as L
    from pvvc.icp import IcpBatch, make_pairs, rotation_error_deg

    pairs = make_pairs(64, seed=21)
    b = IcpBatch(pairs)
    kw = dict(max_corr_dist=1e6, max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
    b.run(**kw)
    T0, m0, i0, c0 = b.results()
    prm = L.IcpParams(kw["max_corr_dist"], kw["max_iter"], kw["fitness_eps"], kw["transform_eps"], kw["mse_abs_eps"])
    centroids = np.array([s.mean(0) for s in pairs.src])
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        T = torch.full((b.n, 16), float("nan"), dtype=torch.float32, device="cuda")
        mse = torch.full((b.n,), -7.0, dtype=torch.float32, device="cuda")
        iters = torch.zeros(b.n, dtype=torch.int32, device="cuda")
        conv = torch.zeros(b.n, dtype=torch.uint8, device="cuda")
        assert _call_noalloc(pvvc_lib, b, prm, T, mse, iters, conv) == 0
        torch.cuda.synchronize()
        T1 = T.cpu().numpy().reshape(-1, 4, 4)
        m1 = mse.cpu().numpy()
        assert np.isfinite(T1).all()
        assert (rotation_error_deg(T1, T0) < ROT_TOL_DEG).all()
        p0 = np.einsum("nij,nj->ni", T0[:, :3, :3], centroids) + T0[:, :3, 3]
        p1 = np.einsum("nij,nj->ni", T1[:, :3, :3], centroids) + T1[:, :3, 3]
        assert (np.linalg.norm(p0 - p1, axis=1) < TRANS_TOL_VOX).all()
        assert (np.abs(m1 - m0) <= MSE_RTOL * m0 + 1e-3).all()
        assert np.array_equal(conv.cpu().numpy().astype(bool), c0)


def test_icp_noalloc_rejects_batches_beyond_its_scratch(pvvc_lib):
    import torch
    from pvvc import _lib as L
    from pvvc.icp import IcpBatch, make_pairs

    b = IcpBatch(make_pairs(2, seed=3))
    prm = L.IcpParams(1e6, 10, 0.0, 0.0, 1e-6)
    T = torch.zeros((b.n, 16), dtype=torch.float32, device="cuda")
    mse = torch.zeros(b.n, dtype=torch.float32, device="cuda")
    iters = torch.zeros(b.n, dtype=torch.int32, device="cuda")
    conv = torch.zeros(b.n, dtype=torch.uint8, device="cuda")
    assert _call_noalloc(pvvc_lib, b, prm, T, mse, iters, conv, npairs=513) == 11   # PVVC_ERR_CAPACITY
    lib = pvvc_lib.lib()
    rc = lib.pvvc_icp_batch_noalloc(b.n, b.src.data_ptr(), b.soff.data_ptr(), b.tgt.data_ptr(), b.toff.data_ptr(), None,
                                    C.byref(prm), T.data_ptr(), mse.data_ptr(), iters.data_ptr(), conv.data_ptr(),
                                    (1 << 20) + 1, torch.cuda.current_stream().cuda_stream)
    assert rc == 11
