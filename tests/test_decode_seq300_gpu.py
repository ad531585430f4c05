"""Decode parity at the full-size workload the headline throughput is quoted
on: one whole GoP of the seq300 sequence (30 frames of ~800k points on the
10-bit grid, ~470 patches per frame with lognormal sizes up to 8,000 points,
octrees 10-11 levels deep) at every quantisation step of the sweep
{4, 8, 16, 32}.  The GPU decodes it with the autotuned launch shapes, with
the long-slice RLGR split forced on, and with a three-tier split, through
pvvc_decode and through a CUDA-graph replay; geometry (uint32 view) and
colours must equal the oracle's restatement of the reference CPU decoder
(invert_raht_octree.cc:22-120, pvvc_decompression.cc:141-150) bit for bit.
Every group here (the 30 frames of a patch) is a window group: the long
tier's slices are decoded one thread per slice, the others by the windowed
RLGR, a warp per group."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def _oracle_gop(oracle, pvvc, frames):
    decs = [oracle.decoder() for _ in range(4096)]
    xs, rs = [], []
    for b in frames:
        x, r, st = oracle.decode_frame(decs, pvvc.parse_frame(b), nthreads=os.cpu_count() or 4)
        assert (st == 0).all()
        xs.append(x)
        rs.append(r)
    return np.concatenate(xs), np.concatenate(rs)


def _decode(torch, pvvc, batch, dec, pay, tune, graph=False):
    plan = pvvc.Plan(batch, tune=tune)
    P = plan.total_points
    xyz = torch.zeros((P, 3), dtype=torch.float32, device="cuda")
    rgb = torch.zeros((P, 3), dtype=torch.uint8, device="cuda")
    st = torch.full((batch.nslices,), -1, dtype=torch.int32, device="cuda")
    ws = torch.empty(plan.workspace_bytes, dtype=torch.uint8, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    if graph:
        g = plan.graph(dec, pay.data_ptr(), xyz.data_ptr(), rgb.data_ptr(), 0, st.data_ptr(), ws.data_ptr(), ws.numel())
        g.launch(sp)
        g.launch(sp)  # a replay over a state the first one left must give the same bytes
    else:
        plan.decode(dec, pay.data_ptr(), xyz.data_ptr(), rgb.data_ptr(), 0, st.data_ptr(), ws.data_ptr(), ws.numel(), sp)
    torch.cuda.synchronize()
    return xyz.cpu().numpy(), rgb.cpu().numpy(), st.cpu().numpy(), plan.info()


@pytest.mark.parametrize("qp", [4, 8, 16, 32])
def test_seq300_gop_bit_exact(pvvc_lib, oracle, torch, qp):
    pvvc = pvvc_lib
    s = pvvc.Synth(pvvc.config("seq300", nframes=30, qp_i=qp, qp_p=qp, seed=40 + qp))
    frames = s.frames()
    parsed = [pvvc.parse_frame(b) for b in frames]
    sizes = np.concatenate([f.size for f in parsed])
    assert sizes.max() > 4500 and len(parsed) == 30  # the lognormal tail is present
    batch = pvvc.pack_frames(parsed)
    stride = max(int(f.index.max()) + 1 for f in parsed)
    dec = pvvc.Decoder(nslots=stride, max_leaves=8192, max_nodes=16384)
    pay = torch.from_numpy(batch.payload).to("cuda")
    want_xyz, want_rgb = _oracle_gop(oracle, pvvc, frames)
    assert want_xyz.shape[0] == batch.points

    auto, _ = pvvc.autotune(batch, dec, pay.data_ptr(), reps=1, stream=torch.cuda.current_stream().cuda_stream)
    shapes = [
        (auto, True),                                     # the autotuner's pick, graph replay
        ((3, 4, 64, 64, -1, 32), False),                  # long-slice split (128 x 64 slices), no medium tier
        ((2, 8, 128, 16, 30, 16), True),                  # three tiers, 16 lanes per long warp
    ]
    for tune, graph in shapes:
        xyz, rgb, st, info = _decode(torch, pvvc, batch, dec, pay, tune, graph)
        assert (st == 0).all(), (tune, np.unique(st))
        # every group holds the 30 frames of a patch: all but the long tier's go to the windowed RLGR, which writes
        # every coefficient itself, so only the long tier's planes (the largest patches) are cleared -- less than
        # all of them (3 planes x 32 lanes x 4 bytes per leaf of each group's tree)
        full = 384 * int(batch.size[(batch.type & 0x02) == 0].astype(np.int64).sum())
        assert 0 < info["clear_bytes"] < full, (info["clear_bytes"], full)
        if tune is not auto:
            assert info["tune"]["rlgr_long_ctas"] > 0
        bad = np.flatnonzero((xyz.view(np.uint32) != want_xyz.view(np.uint32)).any(1))
        assert bad.size == 0, (tune, "geometry differs", bad[:8])
        bad = np.flatnonzero((rgb != want_rgb).any(1))
        assert bad.size == 0, (tune, "colours differ", bad[:8], rgb[bad[:4]], want_rgb[bad[:4]])
