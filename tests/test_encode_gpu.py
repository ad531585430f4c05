"""GPU encoder back end (pvvc_encode_colors: forward RAHT, quantisation,
RLGR on the device) against the CPU encoder (pvvc_encode_patch_gop), whose
bytes the CPU tests pin to the reference's own encoder: every colour payload
must be byte-identical.  The GPU-encoded GoP then decodes, on the GPU, to the
oracle's decode of the same bytes."""
import numpy as np
import pytest

from conftest import rgb_matches
from test_decode_gpu import _dev, decode_batch, oracle_decode

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def _edge_patches(rng, nframes):
    pats = [np.array([[100.0, 200.0, 300.0]], np.float32),
            np.array([[0.0, 0.0, 0.0], [37.0, 5.0, 90.0]], np.float32),
            (np.stack(np.meshgrid(np.arange(8), np.arange(8), np.arange(8), indexing="ij"), -1).reshape(-1, 3) + 40)
            .astype(np.float32)]
    p = rng.integers(0, 20, (300, 3)).astype(np.float32) + np.float32(0.5)
    pats.append(np.concatenate([p, p[:60]]))  # shared voxels: leaves average colours
    out = []
    for xyz in pats:
        yuv = [rng.uniform(0, 255, (xyz.shape[0], 3)).astype(np.float32)]
        yuv += [rng.normal(0, 40, (xyz.shape[0], 3)).astype(np.float32) for _ in range(nframes - 1)]
        out.append((xyz, np.stack(yuv)))
    return out


def _gop(pvvc_lib, patches, qps):
    """Frames of one GoP with geometry only (colour payloads to be encoded),
    the leaf signal per slice in batch order, and the CPU encoder's payloads."""
    nf = len(qps)
    geos, leaves, cpu = [], [], []
    for xyz, yuv in patches:
        geo, nl, leaf = pvvc_lib.patch_leaf_yuv(xyz, yuv)
        g2, nl2, cols = pvvc_lib.encode_patch_gop(xyz, yuv, qps)
        assert g2 == geo and nl2 == nl
        geos.append((geo, nl))
        leaves.append(leaf)
        cpu.append(cols)
    P = len(patches)
    frames = []
    for f in range(nf):
        frames.append(pvvc_lib.Frame(f, np.arange(P, dtype=np.int32), np.full(P, 1 if f == 0 else 3, np.uint8),
                                     np.array([g[1] for g in geos], np.uint32), np.full(P, qps[f], np.uint8),
                                     np.tile(np.eye(4, dtype=np.float32).reshape(16), (P, 1)),
                                     [g[0] if f == 0 else b"" for g in geos], [b""] * P))
    batch = pvvc_lib.pack_frames(frames)
    leaf_yuv = np.zeros((max(batch.points, 1), 3), np.float32)
    k = 0
    for f in range(nf):
        for p in range(P):
            o = int(batch.out_off[k])
            leaf_yuv[o:o + geos[p][1]] = leaves[p][f]
            k += 1
    return frames, batch, leaf_yuv, cpu


def _encode(pvvc_lib, torch, batch, leaf_yuv, nslots):
    dec = pvvc_lib.Decoder(nslots=nslots, max_leaves=8192)
    enc = pvvc_lib.Encoder()
    cap = ((16 * batch.size.astype(np.uint64) + 64 + 3) // 4 * 4).astype(np.uint32)
    off = np.concatenate([[0], np.cumsum(cap.astype(np.uint64))[:-1]]).astype(np.uint64)
    pay = _dev(torch, batch.payload)
    ly = _dev(torch, leaf_yuv)
    out = torch.zeros(int(cap.astype(np.uint64).sum()) + 16, dtype=torch.uint8, device="cuda")
    olen = torch.zeros(batch.nslices, dtype=torch.int32, device="cuda")
    st = torch.full((batch.nslices,), -1, dtype=torch.int32, device="cuda")
    enc.encode(batch, dec, pay.data_ptr(), ly.data_ptr(), out.data_ptr(), off, cap, olen.data_ptr(), st.data_ptr(),
               torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    lens = olen.cpu().numpy().astype(np.int64)
    return [o[int(off[k]):int(off[k]) + lens[k]].tobytes() for k in range(batch.nslices)], st.cpu().numpy()


@pytest.mark.parametrize("qps", [[10, 30, 30, 30], [4, 4, 8, 16], [32, 32, 32, 32]])
def test_gpu_encoder_bytes_equal_cpu_encoder(pvvc_lib, torch, qps):
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", nframes=4, gof=4, seed=13))
    patches = [s.patch(0, p)[:2] for p in range(s.patch_count(0))]
    patches += _edge_patches(np.random.default_rng(5), len(qps))
    frames, batch, leaf_yuv, cpu = _gop(pvvc_lib, patches, qps)
    got, st = _encode(pvvc_lib, torch, batch, leaf_yuv, len(patches))
    assert (st == 0).all(), st
    k = 0
    for f in range(len(qps)):
        for p in range(len(patches)):
            assert got[k] == cpu[p][f], (f, p, len(got[k]), len(cpu[p][f]))
            k += 1


def test_gpu_encoded_gop_decodes_like_the_oracle(pvvc_lib, oracle, torch):
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", nframes=4, gof=4, seed=17))
    patches = [s.patch(0, p)[:2] for p in range(s.patch_count(0))]
    qps = [10, 30, 30, 30]
    frames, batch, leaf_yuv, _ = _gop(pvvc_lib, patches, qps)
    got, st = _encode(pvvc_lib, torch, batch, leaf_yuv, len(patches))
    assert (st == 0).all()
    k = 0
    for fr in frames:
        for i in range(fr.n):
            fr.color[i] = got[k]
            k += 1
    enc_bytes = [pvvc_lib.write_frame(fr) for fr in frames]
    dec = pvvc_lib.Decoder(nslots=len(patches), max_leaves=8192)
    xyz, rgb, dst = decode_batch(torch, pvvc_lib, dec, pvvc_lib.pack_frames([pvvc_lib.parse_frame(b) for b in enc_bytes]))
    assert (dst == 0).all()
    ref = oracle_decode(oracle, pvvc_lib, enc_bytes, len(patches))
    ox = np.concatenate([r[0] for r in ref])
    orgb = np.concatenate([r[1] for r in ref])
    oyuv = np.concatenate([r[3] for r in ref])
    assert np.array_equal(xyz.view(np.uint32), ox.view(np.uint32))
    assert rgb_matches(rgb, orgb, oyuv).all()


def test_gpu_encoder_reports_capacity(pvvc_lib, torch):
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", nframes=2, gof=2, seed=19))
    patches = [s.patch(0, p)[:2] for p in range(4)]
    frames, batch, leaf_yuv, _ = _gop(pvvc_lib, patches, [4, 4])
    dec = pvvc_lib.Decoder(nslots=4, max_leaves=8192)
    enc = pvvc_lib.Encoder()
    cap = np.full(batch.nslices, 8, np.uint32)  # far too small
    off = (np.arange(batch.nslices, dtype=np.uint64) * 8).astype(np.uint64)
    pay = _dev(torch, batch.payload)
    ly = _dev(torch, leaf_yuv)
    out = torch.zeros(8 * batch.nslices + 16, dtype=torch.uint8, device="cuda")
    olen = torch.zeros(batch.nslices, dtype=torch.int32, device="cuda")
    st = torch.full((batch.nslices,), -1, dtype=torch.int32, device="cuda")
    enc.encode(batch, dec, pay.data_ptr(), ly.data_ptr(), out.data_ptr(), off, cap, olen.data_ptr(), st.data_ptr(),
               torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert (st.cpu().numpy() == 11).all() and (olen.cpu().numpy() == 0).all()
