"""pvvc_icp_batch_noalloc: the registration entry point for callers that cannot
allocate device memory (a host application that owns the GPU's memory, a
per-frame callback that must not synchronise the device).  It must give the
results of pvvc_icp_batch -- within the ICP tests' tolerance -- on two calls
in a row, also with its fixed scratch filled to the last point, refuse
batches beyond that scratch, and keep a caller that understates the target
point count from writing past it.  Collected last on purpose so that a run
stopping at the first failure has run everything else."""
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


def _bufs(torch, n):
    return (torch.full((n, 16), float("nan"), dtype=torch.float32, device="cuda"),
            torch.full((n,), -7.0, dtype=torch.float32, device="cuda"),
            torch.zeros(n, dtype=torch.int32, device="cuda"), torch.zeros(n, dtype=torch.uint8, device="cuda"))


def test_icp_noalloc_at_its_exact_capacity(pvvc_lib):
    """512 pairs whose targets hold exactly 1,048,576 points: every offset
    region of the fixed array is used up to its last entry."""
    import torch
    from pvvc import _lib as L
    from pvvc.icp import IcpBatch, Pairs, make_pairs

    base = make_pairs(512, seed=5)
    rng = np.random.default_rng(9)
    tgt = []
    for q in base.tgt:  # every target resized to 2048 points: 512 x 2048 = 1 << 20
        if q.shape[0] >= 2048:
            tgt.append(q[rng.choice(q.shape[0], 2048, replace=False)])
        else:
            lo, hi = q.min(0), q.max(0)
            tgt.append(np.concatenate([q, rng.uniform(lo, hi, (2048 - q.shape[0], 3)).astype(np.float32)]))
    pairs = Pairs(base.src, tgt, base.T_true)
    b = IcpBatch(pairs)
    assert b.n == 512 and b.nt == 1 << 20
    kw = dict(max_corr_dist=1e6, max_iter=20, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
    b.run(**kw)
    T0, m0, _, c0 = b.results()
    prm = L.IcpParams(kw["max_corr_dist"], kw["max_iter"], kw["fitness_eps"], kw["transform_eps"], kw["mse_abs_eps"])
    code = C.c_int32(0)
    assert pvvc_lib.lib().pvvc_device_error_take(C.byref(code)) == 0
    for _ in range(2):
        T, mse, iters, conv = _bufs(torch, b.n)
        assert _call_noalloc(pvvc_lib, b, prm, T, mse, iters, conv) == 0
        torch.cuda.synchronize()
        # the same kernels on the same inputs as pvvc_icp_batch: the same results
        assert np.array_equal(T.cpu().numpy().reshape(-1, 4, 4), T0)
        assert np.array_equal(mse.cpu().numpy(), m0)
        assert np.array_equal(conv.cpu().numpy().astype(bool), c0)
        assert pvvc_lib.lib().pvvc_device_error_take(C.byref(code)) == 0 and code.value == 0


def test_icp_noalloc_understated_total_stays_inside_its_array(pvvc_lib):
    """A caller that passes a total_tgt_points below tgt_off[npairs]: the host
    check cannot see it, the kernels do.  The pair whose targets lie past the
    array's capacity gets NaN results and PVVC_ERR_CAPACITY through
    pvvc_device_error_take; the pair inside it is registered as usual; a
    following correct call is unaffected."""
    import torch
    from pvvc import _lib as L
    from pvvc.icp import IcpBatch, Pairs, make_pairs

    base = make_pairs(2, seed=13)
    rng = np.random.default_rng(4)
    big = base.tgt[0]
    lo, hi = big.min(0), big.max(0)
    pad = rng.uniform(lo - 200, hi + 200, ((1 << 20) - 100 - big.shape[0], 3)).astype(np.float32)
    tgt = [np.concatenate([big, pad]), base.tgt[1]]  # pair 1 (> 200 points) ends past 1 << 20
    b = IcpBatch(Pairs(base.src, tgt, base.T_true))
    assert b.nt > 1 << 20 and int(b.toff[1].item()) < 1 << 20
    prm = L.IcpParams(1e6, 5, 0.0, 0.0, 1e-6)
    code = C.c_int32(0)
    assert pvvc_lib.lib().pvvc_device_error_take(C.byref(code)) == 0
    T, mse, iters, conv = _bufs(torch, b.n)
    lib = pvvc_lib.lib()
    rc = lib.pvvc_icp_batch_noalloc(b.n, b.src.data_ptr(), b.soff.data_ptr(), b.tgt.data_ptr(), b.toff.data_ptr(), None,
                                    C.byref(prm), T.data_ptr(), mse.data_ptr(), iters.data_ptr(), conv.data_ptr(), 1000,
                                    torch.cuda.current_stream().cuda_stream)
    assert rc == 0  # the host cannot tell
    torch.cuda.synchronize()
    assert lib.pvvc_device_error_take(C.byref(code)) == 0 and code.value == 11  # PVVC_ERR_CAPACITY
    Tn = T.cpu().numpy()
    assert np.isnan(Tn[1]).all() and np.isnan(mse.cpu().numpy()[1]) and int(iters.cpu()[1]) == 0
    assert np.isfinite(Tn[0]).all() and int(iters.cpu()[0]) > 0
    # a correct call afterwards: as pvvc_icp_batch, and no error
    good = IcpBatch(make_pairs(8, seed=2))
    good.run(max_corr_dist=1e6, max_iter=5, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
    T0 = good.results()[0]
    T, mse, iters, conv = _bufs(torch, good.n)
    assert _call_noalloc(pvvc_lib, good, prm, T, mse, iters, conv) == 0
    torch.cuda.synchronize()
    assert np.array_equal(T.cpu().numpy().reshape(-1, 4, 4), T0)
    assert lib.pvvc_device_error_take(C.byref(code)) == 0 and code.value == 0
