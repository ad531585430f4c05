"""The GoP encode flow with registration (PatchFitting::AddPatch +
GoPEncoding::Encode, src/patch/patch_fitting.cc:34-90, GoP_encoding.cc:
120-205) end to end on the GPU, on one GoP of the config-1 workload (8 frames,
~64 patches, 9-bit grid): registration, colour interpolation, RAHT/RLGR
encoding, decoding and PSNR against the source frames.  The bitstream it
writes must decode identically through the oracle (the reference decoder's
restatement), and registering with plain ICP must come close to encoding with
the generator's true motion."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def flow(pvvc_lib):
    import torch
    assert torch.cuda.is_available()
    from pvvc import encode_flow
    s = pvvc_lib.Synth(pvvc_lib.config("gof8", seed=21))
    return encode_flow, encode_flow.GopSource(s, 0, seed=1)


def test_encode_flow_true_motion_and_plain_icp(flow):
    ef, src = flow
    truth = ef.encode_decode_gop(src, None, qp=8)
    plain = ef.encode_decode_gop(src, ef.register_plain, qp=8, fitting_ths=50.0)
    for r in (truth, plain):
        assert r["frames"] == 8 and np.isfinite(r["psnr_y"]) and r["psnr_y"] > 25
        assert r["bits_per_point"] > 0
    # frame 0 is coded without motion: the same geometry in both
    assert truth["psnr_geo_per_frame"][0] == plain["psnr_geo_per_frame"][0]
    # registered motion: geometry within 2 dB of the true motion's
    assert plain["psnr_geo"] > truth["psnr_geo"] - 2.0
    assert plain["fitting_gate_pass"] is not None and plain["fitting_gate_pass"] > 0.9


def test_encode_flow_bitstream_decodes_identically_in_the_oracle(flow, oracle, pvvc_lib):
    ef, src = flow
    r = ef.encode_decode_gop(src, ef.register_plain, qp=8, keep_frames=True)
    frames = r["frame_bytes"]
    dec = pvvc_lib.Decoder(nslots=src.npatch, max_leaves=8192, max_nodes=16384)
    xyz, rgb, st = dec.decode_frames(frames)
    assert (st == 0).all()
    decs = [oracle.decoder() for _ in range(src.npatch)]
    off = 0
    for b in frames:
        ox, orgb, ost = oracle.decode_frame(decs, pvvc_lib.parse_frame(b), nthreads=4)
        assert (ost == 0).all()
        n = ox.shape[0]
        assert np.array_equal(xyz[off:off + n].view(np.uint32), ox.view(np.uint32))
        assert np.array_equal(rgb[off:off + n], orgb)
        off += n
