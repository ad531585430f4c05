"""Batched GPU ICP against the oracle's restatement of the reference's PCL
point-to-point ICP (parity is unpinned against PCL itself, which is not
available): transforms agree within a stated rotation / translation
tolerance and the registration MSE agrees to 2 % (FP32 nearest neighbours
and Kahan-compensated FP32 sums on the GPU, FP64 throughout in the oracle)."""
import numpy as np
import pytest

ROT_TOL_DEG = 0.1      # GPU vs oracle final rotation
TRANS_TOL_VOX = 0.1    # GPU vs oracle final translation, at the source centroid
MSE_RTOL = 0.02        # GPU vs oracle fitness score


def _pairs(pvvc_lib, n, seed):
    from pvvc.icp import make_pairs
    return make_pairs(n, seed=seed)


def _trans_err(A, B, pairs):
    c = np.array([s.mean(0) for s in pairs.src])
    pa = np.einsum("nij,nj->ni", A[:, :3, :3], c) + A[:, :3, 3]
    pb = np.einsum("nij,nj->ni", B[:, :3, :3], c) + B[:, :3, 3]
    return np.linalg.norm(pa - pb, axis=1)


def test_oracle_icp_recovers_ground_truth(pvvc_lib, oracle):
    from pvvc.icp import rotation_error_deg
    pairs = _pairs(pvvc_lib, 6, 1)
    Ts, fits = [], []
    for s, t in zip(pairs.src, pairs.tgt):
        T, fit, it, conv = oracle.icp_align(s, t, max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
        assert conv  # the iteration cap counts as converged, as in PCL
        Ts.append(T)
        fits.append(fit)
    err = rotation_error_deg(np.array(Ts), pairs.T_true)
    # plain ICP from identity can stop in a local minimum; most pairs register
    assert np.median(err) < 0.5 and (np.array(fits) < 2.0).sum() >= 4


def test_oracle_cloud_mse_identity_is_zero(oracle):
    rng = np.random.default_rng(0)
    a = rng.integers(0, 100, (500, 3)).astype(np.float32)
    assert oracle.cloud_mse(a, a) == 0.0
    b = a + np.float32(1.0)
    assert abs(oracle.cloud_mse(a, b) - 3.0) < 1e-5 or oracle.cloud_mse(a, b) <= 3.0


CLOUD_MSE_RTOL = 1e-5  # the reference sums float distances in point order; the oracle (double) and GPU (compensated) do not


def _cloud_mse_golden():
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "cloud_mse.npz"))
    ao, bo = z["a_off"], z["b_off"]
    return [(z["a"][ao[i]:ao[i + 1]], z["b"][bo[i]:bo[i + 1]], float(z["mse"][i])) for i in range(len(z["mse"]))]


def test_oracle_cloud_mse_matches_reference(oracle):
    """Pinned against the reference's own ICPBase::CloudMSE (golden fixture
    from tests/golden/make_golden.py)."""
    for a, b, want in _cloud_mse_golden():
        got = oracle.cloud_mse(a, b)
        assert abs(got - want) <= CLOUD_MSE_RTOL * want, (got, want)


@pytest.mark.gpu
def test_gpu_cloud_mse_matches_reference(pvvc_lib):
    import torch
    from pvvc.icp import IcpBatch, Pairs
    cases = _cloud_mse_golden()
    b = IcpBatch(Pairs([c[0] for c in cases], [c[1] for c in cases], np.repeat(np.eye(4)[None], len(cases), 0)))
    T = torch.from_numpy(np.tile(np.eye(4, dtype=np.float32).reshape(16), (len(cases), 1))).cuda()
    got = b.cloud_mse(T)
    for i, (_, _, want) in enumerate(cases):
        assert abs(got[i] - want) <= CLOUD_MSE_RTOL * want, (i, got[i], want)


@pytest.mark.gpu
def test_gpu_icp_matches_oracle(pvvc_lib, oracle):
    import torch
    assert torch.cuda.is_available()
    from pvvc.icp import IcpBatch, rotation_error_deg
    pairs = _pairs(pvvc_lib, 48, 3)
    b = IcpBatch(pairs)
    b.run(max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
    T, mse, iters, conv = b.results()
    To, mo = [], []
    for s, t in zip(pairs.src, pairs.tgt):
        Tt, fit, it, cv = oracle.icp_align(s, t, max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
        To.append(Tt)
        mo.append(fit)
    To, mo = np.array(To), np.array(mo)
    assert conv.all()
    rot = rotation_error_deg(T, To)
    tr = _trans_err(T, To, pairs)
    assert (rot < ROT_TOL_DEG).mean() >= 0.95, rot
    assert (tr < TRANS_TOL_VOX).mean() >= 0.95, tr
    assert (np.abs(mse - mo) <= MSE_RTOL * mo + 1e-3).mean() >= 0.95, (mse, mo)


@pytest.mark.gpu
def test_gpu_cloud_mse_matches_oracle(pvvc_lib, oracle):
    import torch
    from pvvc.icp import IcpBatch
    pairs = _pairs(pvvc_lib, 16, 4)
    b = IcpBatch(pairs)
    T = torch.from_numpy(np.ascontiguousarray(pairs.T_true.reshape(-1, 16), np.float32)).cuda()
    got = b.cloud_mse(T)
    for i, (s, t) in enumerate(zip(pairs.src, pairs.tgt)):
        M = pairs.T_true[i].astype(np.float32)
        st = (s @ M[:3, :3].T + M[:3, 3]).astype(np.float32)
        want = oracle.cloud_mse(st, t)
        assert abs(got[i] - want) <= 1e-3 * want + 1e-4, (i, got[i], want)


@pytest.mark.gpu
def test_gpu_icp_edge_cases(pvvc_lib):
    """Tiny and degenerate pairs finish with a status instead of hanging."""
    import torch
    from pvvc.icp import IcpBatch, Pairs
    rng = np.random.default_rng(5)
    one = np.array([[1.0, 2.0, 3.0]], np.float32)
    two = np.array([[0, 0, 0], [5, 0, 0]], np.float32)
    line = np.stack([np.arange(50), np.zeros(50), np.zeros(50)], 1).astype(np.float32)
    cloud = rng.integers(0, 40, (300, 3)).astype(np.float32)
    pairs = Pairs([one, two, line, cloud], [one + 1, two, line + 2, cloud + 0.5], np.repeat(np.eye(4)[None], 4, 0))
    b = IcpBatch(pairs)
    b.run(max_iter=30)
    T, mse, iters, conv = b.results()
    assert not conv[0] and not conv[1]          # fewer than 3 correspondences
    assert np.isfinite(T).all() and (iters <= 30).all()
    assert conv[3] and mse[3] < 1.0
