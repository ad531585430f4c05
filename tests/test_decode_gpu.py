"""GPU decode path (libpvvc_gb300.so on cuda:0) against the oracle and the
reference's golden outputs.  Geometry must be bit-identical; colours must
equal the reference's wherever its uint8 cast is defined (see
conftest.rgb_matches), which makes them bit-identical in practice."""
import ctypes
import ctypes.util
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_expected, golden_frames, rgb_matches

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def _dev(torch, a: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def decode_batch(torch, pvvc, dec, batch, points24=False, tune=None):
    """Plan + pvvc_decode through the C ABI with torch-allocated buffers."""
    plan = pvvc.Plan(batch, tune=tune)
    P = max(plan.total_points, 1)
    pay = _dev(torch, batch.payload)
    xyz = torch.zeros((P, 3), dtype=torch.float32, device="cuda")
    rgb = torch.zeros((P, 3), dtype=torch.uint8, device="cuda")
    p24 = torch.zeros((P, 6), dtype=torch.float32, device="cuda") if points24 else None
    st = torch.full((max(batch.nslices, 1),), -1, dtype=torch.int32, device="cuda")
    ws = torch.empty(max(plan.workspace_bytes, 256), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    plan.decode(dec, pay.data_ptr(), xyz.data_ptr(), rgb.data_ptr(), p24.data_ptr() if points24 else 0, st.data_ptr(),
                ws.data_ptr(), ws.numel(), stream)
    torch.cuda.synchronize()
    out = (xyz.cpu().numpy()[:plan.total_points], rgb.cpu().numpy()[:plan.total_points], st.cpu().numpy()[:batch.nslices])
    if points24:
        out = out + (p24.cpu().numpy()[:plan.total_points],)
    return out


def oracle_decode(oracle, pvvc, frames, ndec):
    decs = [oracle.decoder() for _ in range(ndec)]
    res = []
    for b in frames:
        fr = pvvc.parse_frame(b)
        xyz, rgb, st = oracle.decode_frame(decs, fr, nthreads=4)
        # per-slice YUV for the colour rule, in frame order
        yuv = np.concatenate([decs[int(i)].get_patch()[1] for i in fr.index]) if fr.n else np.zeros((0, 3), np.float32)
        res.append((xyz, rgb, st, yuv))
    return res


def test_golden_gop_host_api(pvvc_lib, oracle, torch):
    exp = golden_expected()
    frames = golden_frames("raw")
    ref = oracle_decode(oracle, pvvc_lib, frames, 8)
    dec = pvvc_lib.Decoder(nslots=16, max_leaves=4096)
    # the whole GoP in one call, then again frame by frame (state persists)
    xyz, rgb, st = dec.decode_frames(frames)
    assert (st == 0).all()
    off = 0
    for f in range(4):
        n = exp[f"xyz_{f}"].shape[0]
        assert np.array_equal(xyz[off:off + n].view(np.uint32), exp[f"xyz_{f}"].view(np.uint32))
        assert rgb_matches(rgb[off:off + n], exp[f"rgb_{f}"], ref[f][3]).all()
        off += n
    for f in range(4):
        x1, r1, s1 = dec.decode_frames([frames[f]])
        assert (s1 == 0).all()
        assert np.array_equal(x1.view(np.uint32), exp[f"xyz_{f}"].view(np.uint32))
        assert rgb_matches(r1, exp[f"rgb_{f}"], ref[f][3]).all()


def test_golden_gop_zstd_payloads(pvvc_lib, oracle, torch):
    """The reference encoder's zstd payloads, inflated on the GPU by the host call."""
    exp = golden_expected()
    ref = oracle_decode(oracle, pvvc_lib, golden_frames("raw"), 8)
    dec = pvvc_lib.Decoder(nslots=16, max_leaves=4096)
    xyz, rgb, st = dec.decode_frames(golden_frames("zstd"))
    assert (st == 0).all()
    off = 0
    for f in range(4):
        n = exp[f"xyz_{f}"].shape[0]
        assert np.array_equal(xyz[off:off + n].view(np.uint32), exp[f"xyz_{f}"].view(np.uint32))
        assert rgb_matches(rgb[off:off + n], exp[f"rgb_{f}"], ref[f][3]).all()
        off += n


@pytest.mark.parametrize("qp", [4, 8, 16, 32])
def test_synthetic_gop_device_api_vs_oracle(pvvc_lib, oracle, torch, qp):
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", qp_i=qp, qp_p=qp, seed=qp))
    frames = s.frames()
    parsed = [pvvc_lib.parse_frame(b) for b in frames]
    batch = pvvc_lib.pack_frames(parsed)
    dec = pvvc_lib.Decoder(nslots=128, max_leaves=4096)
    xyz, rgb, st = decode_batch(torch, pvvc_lib, dec, batch)
    assert (st == 0).all()
    ref = oracle_decode(oracle, pvvc_lib, frames, 128)
    for f, (ox, orgb, ost, oyuv) in enumerate(ref):
        a, b = batch.frame_first_point[f], batch.frame_first_point[f + 1]
        assert (ost == 0).all()
        assert np.array_equal(xyz[a:b].view(np.uint32), ox.view(np.uint32)), f
        assert np.array_equal(rgb[a:b], orgb), f  # oracle colours (clamped) are the product's contract


def test_concurrent_gops_in_one_batch(pvvc_lib, torch):
    s1 = pvvc_lib.Synth(pvvc_lib.config("tiny", seed=1))
    s2 = pvvc_lib.Synth(pvvc_lib.config("tiny", seed=2))
    b1 = pvvc_lib.pack_frames([pvvc_lib.parse_frame(b) for b in s1.frames()])
    b2 = pvvc_lib.pack_frames([pvvc_lib.parse_frame(b) for b in s2.frames()])
    dec = pvvc_lib.Decoder(nslots=256, max_leaves=4096)
    x1, r1, t1 = decode_batch(torch, pvvc_lib, dec, b1)
    x2, r2, t2 = decode_batch(torch, pvvc_lib, dec, b2)
    both = pvvc_lib.concat_batches([b1, b2], slot_stride=128)
    x, r, t = decode_batch(torch, pvvc_lib, dec, both)
    assert (t == 0).all() and (t1 == 0).all() and (t2 == 0).all()
    assert np.array_equal(x, np.concatenate([x1, x2])) and np.array_equal(r, np.concatenate([r1, r2]))


def test_points24_layout_matches_reference_gpu_formula(pvvc_lib, oracle, torch):
    frames = golden_frames("raw")
    ref = oracle_decode(oracle, pvvc_lib, frames, 8)
    batch = pvvc_lib.pack_frames([pvvc_lib.parse_frame(b) for b in frames])
    dec = pvvc_lib.Decoder(nslots=16, max_leaves=4096)
    xyz, rgb, st, p24 = decode_batch(torch, pvvc_lib, dec, batch, points24=True)
    assert (st == 0).all()
    assert np.array_equal(p24[:, :3], xyz)
    f = np.float32
    for fi, (_, _, _, yuv) in enumerate(ref):
        a, b = batch.frame_first_point[fi], batch.frame_first_point[fi + 1]
        y, u, v = yuv[:, 0], yuv[:, 1], yuv[:, 2]
        want = np.stack([(y + f(1.402) * (v - f(128))) / f(255),
                         ((y - f(0.3441) * (u - f(128))) - f(0.7141) * (v - f(128))) / f(255),
                         (y + f(1.772) * (u - f(128))) / f(255)], 1).astype(np.float32)
        # patches under 10 points are painted white (CUDA2OpenGL.cu:54-58)
        sizes = pvvc_lib.parse_frame(frames[fi]).size
        small = np.repeat(sizes < 10, sizes.astype(np.int64))
        want[small] = 1.0
        assert np.array_equal(p24[a:b, 3:], want)


def test_corrupt_and_missing_slices_report_status(pvvc_lib, torch):
    frames = [pvvc_lib.parse_frame(b) for b in golden_frames("raw")]
    f0, f1 = frames[0], frames[1]
    # frame 0: slice 1 colour truncated, slice 2 geometry truncated, slice 3 wrong size, slice 5 invalid type
    f0.color[1] = f0.color[1][: len(f0.color[1]) // 4]
    f0.geometry[2] = f0.geometry[2][:30]
    f0.size = f0.size.copy(); f0.size[3] += 1
    f0.type = f0.type.copy(); f0.type[5] = 0x00
    batch = pvvc_lib.pack_frames([f0])
    dec = pvvc_lib.Decoder(nslots=16, max_leaves=4096)
    _, _, st = decode_batch(torch, pvvc_lib, dec, batch)
    assert st[1] == 2 and st[2] == 3 and st[3] == 4 and st[5] == 6
    assert st[0] == 0 and st[4] == 0 and st[6] == 0 and st[7] == 0
    # predictive slices of the broken patches now lack a reference; a fresh
    # state has no reference at all
    _, _, st1 = decode_batch(torch, pvvc_lib, dec, pvvc_lib.pack_frames([f1]))
    assert st1[0] == 0 and st1[1] == 5 and st1[2] == 5 and st1[3] == 5 and st1[5] == 5
    fresh = pvvc_lib.Decoder(nslots=16, max_leaves=4096)
    _, _, st2 = decode_batch(torch, pvvc_lib, fresh, pvvc_lib.pack_frames([f1]))
    assert (st2 == 5).all()


def test_tree_capacity_is_reported_not_overrun(pvvc_lib, torch):
    frames = [pvvc_lib.parse_frame(b) for b in golden_frames("raw")]
    dec = pvvc_lib.Decoder(nslots=16, max_leaves=600, max_nodes=100000)  # patches above 600 points do not fit
    _, _, st = decode_batch(torch, pvvc_lib, dec, pvvc_lib.pack_frames([frames[0]]))
    big = frames[0].size > 600
    assert (st[big] == 12).all() and (st[~big] == 0).all()


def test_launch_cudaProcess_signature(pvvc_lib, oracle, torch):
    """Reference-signature entry point: device arrays of per-slice pointers,
    24-byte Points output at inner_offset."""
    frames = [pvvc_lib.parse_frame(b) for b in golden_frames("raw")]
    dec = pvvc_lib.Decoder(nslots=16, max_leaves=4096)
    ref_dec = pvvc_lib.Decoder(nslots=16, max_leaves=4096)
    lib = pvvc_lib.lib()
    keep = []
    for fr in frames:
        n = fr.n
        geo = [_dev(torch, np.frombuffer(g or b"\0", np.uint8).copy()) for g in fr.geometry]
        col = [_dev(torch, np.frombuffer(c, np.uint8).copy()) for c in fr.color]
        mvs = [_dev(torch, fr.mv[i].copy()) for i in range(n)]
        keep += geo + col + mvs
        off = np.concatenate([[0], np.cumsum(fr.size.astype(np.int64))[:-1]]).astype(np.int32)
        d = dict(off=_dev(torch, off), idx=_dev(torch, fr.index), typ=_dev(torch, fr.type), size=_dev(torch, fr.size.astype(np.int32)),
                 qp=_dev(torch, fr.qp), gsz=_dev(torch, np.array([len(g) for g in fr.geometry], np.int32)),
                 csz=_dev(torch, np.array([len(c) for c in fr.color], np.int32)),
                 mvp=_dev(torch, np.array([t.data_ptr() for t in mvs], np.int64)),
                 gp=_dev(torch, np.array([t.data_ptr() for t in geo], np.int64)),
                 cp=_dev(torch, np.array([t.data_ptr() for t in col], np.int64)))
        keep += list(d.values())
        P = fr.points
        out = torch.zeros((P, 6), dtype=torch.float32, device="cuda")
        rc = lib.pvvc_launch_cudaProcess(n, 1, out.data_ptr(), fr.timestamp, d["off"].data_ptr(), d["idx"].data_ptr(),
                                         d["typ"].data_ptr(), d["mvp"].data_ptr(), d["size"].data_ptr(), d["qp"].data_ptr(),
                                         d["gp"].data_ptr(), d["gsz"].data_ptr(), d["cp"].data_ptr(), d["csz"].data_ptr(),
                                         dec.h, n, torch.cuda.current_stream().cuda_stream)
        assert rc == 0
        _, _, st, p24 = decode_batch(torch, pvvc_lib, ref_dec, pvvc_lib.pack_frames([fr]), points24=True)
        assert (st == 0).all()
        assert np.array_equal(out.cpu().numpy(), p24)


def test_decode_is_deterministic(pvvc_lib, torch):
    s = pvvc_lib.Synth(pvvc_lib.config("tiny", seed=9))
    batch = pvvc_lib.pack_frames([pvvc_lib.parse_frame(b) for b in s.frames()])
    dec = pvvc_lib.Decoder(nslots=64, max_leaves=4096)
    a = decode_batch(torch, pvvc_lib, dec, batch)
    b = decode_batch(torch, pvvc_lib, dec, batch)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_rlgr_golden_vectors_through_gpu_decode(pvvc_lib, oracle, torch):
    """Every reference-encoded RLGR vector of the fixtures (runs, escapes,
    the lossy >32-bit escape, and escapes taken at k_RP = 0, after which the
    next symbol is read with k_R = 32) decoded as the colour payload of an
    intra slice: status 0, and geometry and colours equal to the oracle's."""
    z = np.load(os.path.join(GOLDEN, "rlgr.npz"))
    so, bo = z["sym_off"], z["byte_off"]
    g = np.stack(np.meshgrid(np.arange(16), np.arange(16), np.arange(16), indexing="ij"), -1).reshape(-1, 3)
    sizes, geos, cols = [], [], []
    for i in range(len(so) - 1):
        sym = z["symbols"][so[i]:so[i + 1]]
        n = max(1, -(-sym.size // 3))
        if sym.size == 3 * n:
            col = z["bytes"][bo[i]:bo[i + 1]].tobytes()           # the reference's own bytes
        else:
            col = oracle.rlgr_encode(np.concatenate([sym, np.zeros(3 * n - sym.size, np.int64)]))
        xyz = (g[:n] * 2 + 3).astype(np.float32)
        geo, nl, _, _ = oracle.encode_patch(xyz, [np.zeros((n, 3), np.float32)], [8])
        assert nl == n
        sizes.append(n); geos.append(geo); cols.append(col)
    m = len(sizes)
    fr = pvvc_lib.Frame(0, np.arange(m, dtype=np.int32), np.full(m, 1, np.uint8), np.array(sizes, np.uint32),
                        np.full(m, 8, np.uint8), np.tile(np.eye(4, dtype=np.float32).reshape(16), (m, 1)), geos, cols)
    dec = pvvc_lib.Decoder(nslots=64, max_leaves=4096)
    xyz, rgb, st = decode_batch(torch, pvvc_lib, dec, pvvc_lib.pack_frames([fr]))
    assert (st == 0).all(), st
    (oxyz, orgb, ost, oyuv), = oracle_decode(oracle, pvvc_lib, [pvvc_lib.write_frame(fr)], m)
    assert (ost == 0).all()
    assert np.array_equal(xyz.view(np.uint32), oxyz.view(np.uint32))
    assert rgb_matches(rgb, orgb, oyuv).all()



def _large_value_frames(pvvc, nframes):
    """Eight patches over `nframes` frames (frame 0 intra), colours and
    residuals uniform in +-scale: at scales far above 255 the dequantised
    coefficients reach far beyond what 8-bit colours give -- at 5e9 with
    step 255 beyond 32 bits, through RLGR's general path (symbols above
    2^23 and raw 32-bit escapes); two patches keep ordinary scales."""
    rng = np.random.default_rng(11)
    specs = [(900, 4.0e4, 2), (900, 5.0e9, 255), (600, 4.0e4, 3), (600, 2.0e5, 1),  # (voxels, scale, step)
             (300, 100.0, 8), (300, 4.0e4, 2), (200, 60.0, 4), (200, 3.0e4, 1)]
    patches = []
    for n, scale, qp in specs:
        pos = rng.choice(64 ** 3, n, replace=False)
        xyz = np.stack([pos // 4096, (pos // 64) % 64, pos % 64], 1).astype(np.float32)
        yuv = rng.uniform(-scale, scale, (nframes, n, 3)).astype(np.float32)
        geo, nl, cols = pvvc.encode_patch_gop(xyz, yuv, [qp] * nframes)
        assert nl == n
        patches.append((geo, nl, cols, qp))
    m = len(patches)
    eye = np.tile(np.eye(4, dtype=np.float32).reshape(16), (m, 1))
    return [pvvc.write_frame(pvvc.Frame(f, np.arange(m, dtype=np.int32), np.full(m, 1 if f == 0 else 3, np.uint8),
                                        np.array([q[1] for q in patches], np.uint32),
                                        np.array([q[3] for q in patches], np.uint8), eye,
                                        [q[0] if f == 0 else b"" for q in patches], [q[2][f] for q in patches]))
            for f in range(nframes)]


@pytest.mark.parametrize("nframes,tune", [(20, None),                         # long tier + windowed RLGR
                                          (20, (3, 4, 64, -1, -1, 32)),       # every group windowed
                                          (8, None),                          # groups below the window size
                                          (3, None)])                         # single slices
def test_large_coefficients_bit_exact(pvvc_lib, oracle, torch, nframes, tune):
    """Very large coefficients decode exactly through every RLGR form and
    both inverse transforms: geometry bit for bit, the unrounded points24
    colours bit for bit against the oracle's YUV, the uint8 colours by the
    reference's cast rule."""
    frames = _large_value_frames(pvvc_lib, nframes)
    parsed = [pvvc_lib.parse_frame(b) for b in frames]
    batch = pvvc_lib.pack_frames(parsed)
    dec = pvvc_lib.Decoder(nslots=16, max_leaves=4096)
    xyz, rgb, st, p24 = decode_batch(torch, pvvc_lib, dec, batch, points24=True, tune=tune)
    assert (st == 0).all(), np.unique(st)
    ref = oracle_decode(oracle, pvvc_lib, frames, 16)
    f = np.float32
    for fi, (ox, orgb, ost, yuv) in enumerate(ref):
        a, b = batch.frame_first_point[fi], batch.frame_first_point[fi + 1]
        assert (ost == 0).all()
        assert np.array_equal(xyz[a:b].view(np.uint32), ox.view(np.uint32)), fi
        y, u, v = yuv[:, 0], yuv[:, 1], yuv[:, 2]
        want = np.stack([(y + f(1.402) * (v - f(128))) / f(255),
                         ((y - f(0.3441) * (u - f(128))) - f(0.7141) * (v - f(128))) / f(255),
                         (y + f(1.772) * (u - f(128))) / f(255)], 1).astype(np.float32)
        assert np.array_equal(p24[a:b, 3:].view(np.uint32), want.view(np.uint32)), fi
        assert rgb_matches(rgb[a:b], orgb, yuv).all(), fi
    assert np.abs(ref[-1][3]).max() > 1e9  # the large scales did reach the decoder

@pytest.mark.parametrize("nframes", [12, 28])
def test_host_call_decodes_gops_in_one_plan_identically(pvvc_lib, torch, nframes):
    """pvvc_decode_frames_host with slots for one region per GoP decodes all
    GoPs of a call together (3 and 7 GoPs, in parts split at GoP boundaries
    whose device-to-host copies overlap the next part's decode); the bytes
    equal run-by-run decoding (a state with one slot per patch), and so does
    the next call, which continues the last GoP from the patch slots."""
    s = pvvc_lib.Synth(pvvc_lib.config("tiny", nframes=nframes, gof=4, seed=21))
    frames = s.frames()
    nidx = max(int(pvvc_lib.parse_frame(b).index.max()) + 1 for b in frames)
    merged = pvvc_lib.Decoder(nslots=(nframes // 4) * nidx, max_leaves=4096)
    serial = pvvc_lib.Decoder(nslots=nidx, max_leaves=4096)
    for part in (frames[:nframes - 1], frames[nframes - 1:]):
        a = merged.decode_frames(part)
        b = serial.decode_frames(part)
        assert (a[2] == 0).all() and (b[2] == 0).all()
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    # a call that starts mid-GoP reads the previous call's state: still run by run
    a = merged.decode_frames(frames[9:11])
    b = serial.decode_frames(frames[9:11])
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_host_call_same_layout_new_content(pvvc_lib, torch):
    """A call whose frames have the layout of the previous call (slots,
    types and sizes) reuses the parts' queue structure and refreshes only
    the per-call fields: new motions and quantisation steps must decode as a
    fresh state decodes them."""
    s = pvvc_lib.Synth(pvvc_lib.config("tiny", nframes=12, gof=4, seed=33))
    frames = s.frames()
    nidx = max(int(pvvc_lib.parse_frame(b).index.max()) + 1 for b in frames)
    rng = np.random.default_rng(3)
    changed = []
    for b in frames:
        f = pvvc_lib.parse_frame(b)
        f.mv = f.mv.copy()
        f.mv[:, 3] += rng.integers(-5, 6, f.n).astype(np.float32)  # new translations
        f.mv[:, 0] *= np.float32(1.5)
        f.qp = np.where(f.qp > 2, f.qp - 1, f.qp + 1).astype(np.uint8)  # new steps, same symbols
        changed.append(pvvc_lib.write_frame(f))
    reused = pvvc_lib.Decoder(nslots=3 * nidx, max_leaves=4096)
    a0 = reused.decode_frames(frames)
    assert (a0[2] == 0).all()
    a = reused.decode_frames(changed)
    fresh = pvvc_lib.Decoder(nslots=3 * nidx, max_leaves=4096)
    b = fresh.decode_frames(changed)
    assert (a[2] == 0).all() and (b[2] == 0).all()
    assert not np.array_equal(a[0], a0[0]) and not np.array_equal(a[1], a0[1])  # the content did change
    for x, y in zip(a, b):
        assert np.array_equal(x, y)



def _gop_frames(pvvc, rng_colour, ngops=3, gof=4):
    """ngops GoPs of gof frames over six patches at fixed positions; the
    colours (and so every colour payload's size) come from rng_colour."""
    pos_rng = np.random.default_rng(5)
    sizes = [700, 500, 300, 200, 120, 60]
    xyzs = []
    for n in sizes:
        pos = pos_rng.choice(32 ** 3, n, replace=False)
        xyzs.append(np.stack([pos // 1024, (pos // 32) % 32, pos % 32], 1).astype(np.float32))
    m = len(sizes)
    frames = []
    for g in range(ngops):
        enc = [pvvc.encode_patch_gop(x, np.concatenate([rng_colour.uniform(0, 255, (1, len(x), 3)),
                                                        rng_colour.uniform(-20, 20, (gof - 1, len(x), 3))]).astype(np.float32),
                                     [8] * gof) for x in xyzs]
        for f in range(gof):
            frames.append(pvvc.write_frame(pvvc.Frame(
                g * gof + f, np.arange(m, dtype=np.int32), np.full(m, 1 if f == 0 else 3, np.uint8),
                np.array([e[1] for e in enc], np.uint32), np.full(m, 8, np.uint8),
                np.tile(np.eye(4, dtype=np.float32).reshape(16), (m, 1)),
                [e[0] if f == 0 else b"" for e in enc], [e[2][f] for e in enc])))
    return frames


def test_host_call_same_layout_new_payloads(pvvc_lib, torch):
    """A second call with the previous call's layout (slots, types, sizes)
    but other colours -- so other payload sizes and offsets -- reuses the
    parts' plans and refreshes their records' per-call fields on the device:
    it must decode as a fresh state does."""
    a = _gop_frames(pvvc_lib, np.random.default_rng(1))
    b = _gop_frames(pvvc_lib, np.random.default_rng(2))
    assert [len(x) for x in a] != [len(x) for x in b]  # the payloads moved
    reused = pvvc_lib.Decoder(nslots=64, max_leaves=4096)
    ra = reused.decode_frames(a)
    rb = reused.decode_frames(b)
    rb2 = reused.decode_frames(b)  # and once more, now from the refreshed records
    fresh = pvvc_lib.Decoder(nslots=64, max_leaves=4096)
    fb = fresh.decode_frames(b)
    assert (ra[2] == 0).all() and (rb[2] == 0).all() and (fb[2] == 0).all()
    assert not np.array_equal(ra[1], rb[1])
    for x, y, z in zip(rb, fb, rb2):
        assert np.array_equal(x, y) and np.array_equal(x, z)

def test_host_call_pinned_and_pageable_outputs_agree(pvvc_lib, torch):
    """Page-locked and pageable output arrays receive the same bytes, for a
    call of several GoPs decoded in parts and for a single-GoP call, and
    nothing is written past the decoded points."""
    s = pvvc_lib.Synth(pvvc_lib.config("tiny", nframes=20, gof=4, seed=5))
    frames = s.frames()
    nidx = max(int(pvvc_lib.parse_frame(b).index.max()) + 1 for b in frames)
    P = sum(pvvc_lib.parse_frame(b).points for b in frames)
    for part in (frames, frames[:4]):
        d1 = pvvc_lib.Decoder(nslots=5 * nidx, max_leaves=4096)
        d2 = pvvc_lib.Decoder(nslots=5 * nidx, max_leaves=4096)
        xp = torch.full((P + 7, 3), -1.0, dtype=torch.float32).pin_memory()
        rp = torch.zeros((P + 7, 3), dtype=torch.uint8).pin_memory()
        x1, r1, s1 = d1.decode_frames(part, out=(xp.numpy(), rp.numpy()))
        x2, r2, s2 = d2.decode_frames(part)
        n = x2.shape[0]
        assert (s1 == 0).all() and (s2 == 0).all() and x1.shape[0] == n
        assert np.array_equal(x1[:n].view(np.uint32), x2.view(np.uint32)) and np.array_equal(r1[:n], r2)
        assert (xp.numpy()[n:] == -1.0).all()  # nothing written past the decoded points


def test_host_call_zstd_sequence_matches_raw(pvvc_lib, torch):
    """A synthetic GoP whose payloads are zstd-compressed by the reference
    encoder's rule (GoP_encoding.cc:158-200: level 22, kept only when smaller)
    decodes exactly as its raw form; a corrupt zstd payload fails the call
    with PVVC_ERR_ZSTD, as the reference's ZstdDecoder throws."""
    import libzstd_ref as zr
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", nframes=8, seed=3))
    raw = s.frames()
    z = [zr.zstd_frame(b, pvvc_lib, 22) for b in raw]
    nz = sum(int(((pvvc_lib.parse_frame(b).type & 0x18) != 0).sum()) for b in z)
    assert nz > 0
    d1 = pvvc_lib.Decoder(nslots=256, max_leaves=4096)
    d2 = pvvc_lib.Decoder(nslots=256, max_leaves=4096)
    x1, r1, s1 = d1.decode_frames(raw)
    x2, r2, s2 = d2.decode_frames(z)
    assert (s1 == 0).all() and (s2 == 0).all()
    assert np.array_equal(x1.view(np.uint32), x2.view(np.uint32)) and np.array_equal(r1, r2)
    t = next(t for t in range(len(z)) if (pvvc_lib.parse_frame(z[t]).type & 0x10).any())
    f = pvvc_lib.parse_frame(z[t])
    i = int(np.flatnonzero(f.type & 0x10)[0])
    c = bytearray(f.color[i])
    c[len(c) // 2] ^= 0xFF
    c[len(c) // 2 + 1] ^= 0x5A
    f.color[i] = bytes(c)
    if zr.decompress(f.color[i], zr.content_size(f.color[i])) is None:
        with pytest.raises(pvvc_lib.PvvcError) as e:
            pvvc_lib.Decoder(nslots=256, max_leaves=4096).decode_frames(z[:t] + [pvvc_lib.write_frame(f)] + z[t + 1:])
        assert e.value.status == 9


def test_host_call_zstd_multi_gop_parts(pvvc_lib, torch):
    """Several GoPs with zstd payloads in one call: the call is decoded in
    parts, each part's payloads inflated ahead of its decode (the first on
    the call's stream, the others on a side stream).  The bytes equal the
    raw frames' and run-by-run decoding; a corrupt zstd payload in the last
    GoP fails the call with PVVC_ERR_ZSTD."""
    import libzstd_ref as zr
    nframes, gof = 24, 4
    raw = pvvc_lib.Synth(pvvc_lib.config("tiny", nframes=nframes, gof=gof, seed=31)).frames()
    z = pvvc_lib.Synth(pvvc_lib.config("tiny", nframes=nframes, gof=gof, seed=31, zstd_level=19)).frames()
    assert sum(int(((pvvc_lib.parse_frame(b).type & 0x18) != 0).sum()) for b in z) > 0
    nidx = max(int(pvvc_lib.parse_frame(b).index.max()) + 1 for b in raw)
    x1, r1, s1 = pvvc_lib.Decoder(nslots=(nframes // gof) * nidx, max_leaves=4096).decode_frames(z)
    x2, r2, s2 = pvvc_lib.Decoder(nslots=nidx, max_leaves=4096).decode_frames(raw)
    assert (s1 == 0).all() and (s2 == 0).all()
    assert np.array_equal(x1.view(np.uint32), x2.view(np.uint32)) and np.array_equal(r1, r2)
    # truncate one zstd payload of the last frame that has one (the declared size stays)
    t = max(t for t in range(nframes) if (pvvc_lib.parse_frame(z[t]).type & 0x18).any())
    assert t >= nframes - gof  # in the last GoP, so in the call's last part
    f = pvvc_lib.parse_frame(z[t])
    i = int(np.flatnonzero(f.type & 0x18)[0])
    if f.type[i] & 0x08:
        f.geometry[i] = bytes(f.geometry[i])[:-2]
    else:
        f.color[i] = bytes(f.color[i])[:-2]
    bad = z[:t] + [pvvc_lib.write_frame(f)] + z[t + 1:]
    dec = pvvc_lib.Decoder(nslots=(nframes // gof) * nidx, max_leaves=4096)
    with pytest.raises(pvvc_lib.PvvcError) as e:
        dec.decode_frames(bad)
    assert e.value.status == 9
