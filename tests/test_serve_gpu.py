"""Playback server (pvvc_server_*): continuous batching across streams must
not change any frame's result.  Each stream is decoded alone and in a mix
with others (arrivals interleaved at random, so batches mix streams and
GoP positions); every frame must be bit-identical in both runs and to the
host decode API (itself pinned to the oracle by the decode tests)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BUDGET = 6 << 30


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


@pytest.fixture(scope="module")
def sequences(pvvc_lib):
    """Three small sequences of two GoPs each, of different sizes."""
    out = []
    for seed, tp in ((21, 3000), (22, 5000), (23, 2000)):
        s = pvvc_lib.Synth(pvvc_lib.config("tiny", seed=seed, nframes=8, gof=4, target_points=tp))
        out.append(s.frames())
    return out


def _server(pvvc_lib, **kw):
    kw.setdefault("max_leaves", 4096)
    kw.setdefault("max_batch_points", 1 << 20)
    kw.setdefault("ring_points", 4 << 20)
    return pvvc_lib.Server(BUDGET, **kw)


def _drain(srv, want, read=True):
    res = {}
    for _ in range(10000):
        if len(res) >= want:
            break
        for c in srv.poll(wait_us=20000):
            res[c["tag"]] = (c["status"],) + (srv.read(c) if read else ())
            srv.release(c)
    assert len(res) == want, (len(res), want)
    return res


def test_each_stream_alone_equals_in_the_mix(pvvc_lib, torch, sequences):
    from pvvc.serve import slots_needed
    alone = {}
    for i, frames in enumerate(sequences):
        srv = _server(pvvc_lib)
        sid = srv.open_stream(slots_needed(frames))
        for k, b in enumerate(frames):
            srv.submit(sid, b, tag=(i, k))
        alone.update(_drain(srv, len(frames)))
        srv.close_stream(sid)
        srv.close()
    # the host API decodes the same bytes (one call per GoP)
    for i, frames in enumerate(sequences):
        dec = pvvc_lib.Decoder(nslots=slots_needed(frames), max_leaves=4096)
        for g in range(0, len(frames), 4):
            xyz, rgb, st = dec.decode_frames(frames[g:g + 4])
            assert (st == 0).all()
            o = 0
            for k in range(g, g + 4):
                s, x, r = alone[(i, k)]
                assert s == 0
                n = x.shape[0]
                assert np.array_equal(x.view(np.uint32), xyz[o:o + n].view(np.uint32)) and np.array_equal(r, rgb[o:o + n])
                o += n
    # the mix: two copies of every stream, submitted in a random interleaving
    rng = np.random.default_rng(5)
    srv = _server(pvvc_lib)
    order = []
    sids = {}
    for copy in range(2):
        for i, frames in enumerate(sequences):
            sids[(copy, i)] = srv.open_stream(slots_needed(frames))
            order += [(copy, i)] * len(frames)
    rng.shuffle(order)
    nxt = {key: 0 for key in sids}
    for key in order:
        copy, i = key
        k = nxt[key]
        nxt[key] += 1
        srv.submit(sids[key], sequences[i][k], tag=(copy, i, k))
    mix = _drain(srv, len(order))
    st = srv.stats()
    srv.close()
    assert st["batches"] >= 1
    for (copy, i, k), (s, x, r) in mix.items():
        s0, x0, r0 = alone[(i, k)]
        assert s == 0 and s0 == 0
        assert np.array_equal(x.view(np.uint32), x0.view(np.uint32)) and np.array_equal(r, r0), (copy, i, k)


def test_admission_by_hbm_budget(pvvc_lib, torch):
    srv = _server(pvvc_lib)
    total = srv.stats()["slots_total"]
    assert total > 4
    half = total // 2 + 1
    a = srv.open_stream(half)
    assert srv.try_open_stream(half) is None  # the budget holds one such stream
    small = srv.open_stream(total - half)     # what is left still admits
    srv.close_stream(a)
    b = srv.try_open_stream(half)
    assert b is not None
    st = srv.stats()
    assert st["slots_free"] == 0 and st["streams_open"] == 2
    assert st["reserved_bytes"] <= BUDGET
    srv.close_stream(small)
    srv.close_stream(b)
    srv.close()


def test_submit_rejects_malformed_frames(pvvc_lib, torch, sequences):
    srv = _server(pvvc_lib)
    sid = srv.open_stream(2)  # fewer slots than the sequence's patch indices
    b = sequences[0][0]
    with pytest.raises(pvvc_lib.PvvcError) as e:
        srv.submit(sid, b[: len(b) // 2])
    assert e.value.status == 10
    with pytest.raises(pvvc_lib.PvvcError) as e:
        srv.submit(sid, b)
    assert e.value.status == 1
    with pytest.raises(pvvc_lib.PvvcError):
        srv.submit(sid + 7, b)
    srv.close()


def test_stream_starting_mid_gop_reports_no_reference(pvvc_lib, torch, sequences):
    from pvvc.serve import slots_needed
    frames = sequences[1]
    srv = _server(pvvc_lib)
    sid = srv.open_stream(slots_needed(frames))
    srv.submit(sid, frames[1], tag="p")   # a predictive frame before any intra frame
    srv.submit(sid, frames[4], tag="i")   # the next GoP's intra frame
    res = _drain(srv, 2, read=False)
    assert res["p"][0] == 5 and res["i"][0] == 0
    srv.close()


def test_small_output_ring_applies_back_pressure(pvvc_lib, torch, sequences):
    from pvvc.serve import slots_needed
    frames = sequences[1]
    biggest = max(pvvc_lib.parse_frame(b).points for b in frames)
    srv = _server(pvvc_lib, max_batch_points=biggest, ring_points=2 * biggest + 1)
    sid = srv.open_stream(slots_needed(frames))
    for k, b in enumerate(frames):
        srv.submit(sid, b, tag=k)
    got = _drain(srv, len(frames))
    ref = pvvc_lib.Decoder(nslots=slots_needed(frames), max_leaves=4096)
    for g in range(0, len(frames), 4):
        xyz, rgb, _ = ref.decode_frames(frames[g:g + 4])
        o = 0
        for k in range(g, g + 4):
            s, x, r = got[k]
            assert s == 0 and np.array_equal(x, xyz[o:o + x.shape[0]]) and np.array_equal(r, rgb[o:o + x.shape[0]])
            o += x.shape[0]
    srv.close()


def test_zstd_frames_served_like_raw(pvvc_lib, torch, sequences):
    """zstd payloads (the reference encoder's rule: level 22, kept when
    smaller) are inflated on the GPU inside the batch: every frame equals the
    raw frame's result; a payload that does not inflate fails its frame
    with PVVC_ERR_ZSTD."""
    import libzstd_ref as zr
    from pvvc.serve import slots_needed
    frames = sequences[1]
    zf = [zr.zstd_frame(b, pvvc_lib, 22) for b in frames]
    assert any((pvvc_lib.parse_frame(b).type & 0x18).any() for b in zf)
    out = {}
    for name, fs in (("raw", frames), ("zstd", zf)):
        srv = _server(pvvc_lib)
        sid = srv.open_stream(slots_needed(fs))
        for k, b in enumerate(fs):
            srv.submit(sid, b, tag=(name, k))
        out.update(_drain(srv, len(fs)))
        srv.close()
    for k in range(len(frames)):
        s0, x0, r0 = out[("raw", k)]
        s1, x1, r1 = out[("zstd", k)]
        assert s0 == 0 and s1 == 0
        assert np.array_equal(x0.view(np.uint32), x1.view(np.uint32)) and np.array_equal(r0, r1)
    # a truncated zstd frame inside a payload: the declared size stays, the inflation fails
    f = pvvc_lib.parse_frame(zf[0])
    i = next(i for i in range(f.n) if f.type[i] & 0x18)
    if f.type[i] & 0x08:
        f.geometry[i] = bytes(f.geometry[i])[:-3]
    else:
        f.color[i] = bytes(f.color[i])[:-3]
    srv = _server(pvvc_lib)
    sid = srv.open_stream(slots_needed(zf))
    srv.submit(sid, pvvc_lib.write_frame(f), tag="bad")
    res = _drain(srv, 1, read=False)
    srv.close()
    assert res["bad"][0] == 9
