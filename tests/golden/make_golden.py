"""Generates the committed golden fixtures from the reference's OWN code.

Run in a checkout that has the reference tree (the build container):
    python tests/golden/make_golden.py
It compiles the reference's sources against the oracle's shim headers
(`make -C oracle ref`) and drives them through oracle/_ref/libpvvc_ref.so:

  rlgr.npz         symbol vectors and RLGREncoder's bytes for them
                   (src/common/entropy_codec.cc:65-159)
  gop/raw_*.frame  a 4-frame GoP (intra + 3 predictive) of 8 patches encoded
                   by RAHTOctree + RLGREncoder (src/octree/raht_octree.cc,
                   GoP_encoding.cc:152-205 quantisation), each slice written
                   by io::SaveSlice and the frame by io::ChangeSliceToFrame
                   (src/io/slice_io.cc:20-322); payloads raw
  gop/zstd_*.frame the same slices with GoPEncoding's zstd-if-smaller
                   (GoP_encoding.cc:158-170,194-204, level 22)
  gop/expected.npz per frame: InvertRAHTOctree::SetSlice/GetPatch output
                   (src/octree/invert_raht_octree.cc:22-120) transformed as
                   pvvc_decompression.cc:141-150 (float32, left to right)
  gop_encode.npz   GoPEncoding::Encode (src/patch/GoP_encoding.cc:97-210)
                   on 4 patches x 3 frames: its k-NN colour interpolation
                   (k = 10; patch_colors_, later frames as residuals), the
                   geometry payload and each frame's colour payload.  The
                   k-d tree is the shim's exact search (lower index first
                   among equal distances).

  cloud_mse.npz    ICPBase::CloudMSE (src/registration/registration_base.cc:
                   114-158) of 6 cloud pairs (its k-d tree the shim's exact
                   search; the sums in float, in point order).

  cloud_quality.npz common::MSE::Compute (src/registration/registration_base.cc:
                   160-223) of 6 coloured cloud pairs: geometric and Y/U/V
                   errors both ways, summed in float as the reference does.

  fitting.npz      PatchFitting::Compute (src/patch/patch_fitting.cc:92-381,
                   direct clustering, the configs' 1.0 / 0.1 / 100) after
                   srand(seed): registered synthetic patch GoPs, and small
                   GoPs of repeated points whose k-means empties clusters and
                   redraws them from rand().

`python tests/golden/make_golden.py gop_encode` (or `cloud_mse`,
`cloud_quality`, `fitting`) writes only that fixture.

Patches: 4 from the seeded synthetic surface generator plus 4 edge cases
(a single point, two distant points, a full 8^3 cube, and points that share
voxels so that leaves average colours).
"""
from __future__ import annotations

import ctypes
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "patchvvc-plus_gb300"))

from oracle import Reference, quantise  # noqa: E402

QP_I, QP_P = 10, 30   # the reference configuration's slice.qp_i / qp_p (test/patchvvc_loot.cfg:36-37)
NFRAMES = 4


def rgb_to_yuv(rgb):
    """ColorYUV(const PointXYZRGB&), include/common/common.h:95-99, float32."""
    f = np.float32
    r, g, b = (rgb[:, i].astype(f) for i in range(3))
    y = r * f(0.299) + g * f(0.587) + b * f(0.114)
    u = r * f(-0.168736) - g * f(0.331264) + b * f(0.5) + f(128)
    v = r * f(0.5) - g * f(0.418688) - b * f(0.081312) + f(128)
    return np.stack([y, u, v], 1).astype(np.float32)


def transform(xyz, m):
    """pvvc_decompression.cc:141-150 in float32, left to right, no fusion."""
    f = np.float32
    x, y, z = xyz[:, 0].astype(f), xyz[:, 1].astype(f), xyz[:, 2].astype(f)
    m = m.astype(f).reshape(4, 4)
    out = np.empty_like(xyz, dtype=f)
    for r in range(3):
        t = x * m[r, 0]
        t = t + y * m[r, 1]
        t = t + z * m[r, 2]
        out[:, r] = t + m[r, 3]
    return out


def rot(axis, deg):
    a = np.asarray(axis, np.float64)
    a /= np.linalg.norm(a)
    th = np.deg2rad(deg)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


def make_rlgr(ref: Reference, rng):
    vecs, kinds = [], []
    for t in range(28):
        n = int(rng.integers(1, 4000))
        k = t % 7
        if k == 0:
            s = rng.integers(-3, 4, n)
        elif k == 1:
            s = np.where(rng.random(n) < 0.9, 0, rng.integers(-50, 51, n))
        elif k == 2:
            s = rng.integers(-100000, 100001, n)
        elif k == 3:
            s = np.where(rng.random(n) < 0.995, 0, rng.integers(-2, 3, n))
        elif k == 4:
            s = np.zeros(n, np.int64)                     # one long run
        elif k == 5:
            s = rng.integers(-(2 ** 31), 2 ** 31, n)      # Golomb-Rice escapes (32-bit raw values)
            s[:: 7] = 0
        else:
            # beyond 32 bits the reference's escape (GRWrite, entropy_codec.cc:59-61)
            # is lossy; the fixture records what its decoder returns
            s = rng.integers(-(2 ** 40), 2 ** 40, n)
            s[:: 7] = 0
        vecs.append(s.astype(np.int64))
        kinds.append(k)
    # kind 7: a Golomb-Rice escape (>= 32 leading ones) taken while k_RP = 0
    # and k_P < 4, so that p = u >> k_R is far above the k_RP cap and the next
    # symbol is read with k_R = 32.  From the initial state (k_P = 0,
    # k_RP = 8) the head -1 -1 -1 0 drives k_RP 8 -> 6 -> 4 -> 2 -> 0 and k_P
    # to 3 (entropy_codec.cc:262-281); |escape| >= 65 makes p >= 129.  Lengths
    # are multiples of 3 (Y|U|V planes).  Own generator, so that the vectors
    # above and the GoP below are unchanged.
    r7 = np.random.default_rng(77)
    for t in range(6):
        head = [-1, -1, -1, 0, int(r7.integers(65, 2 ** 20)) * (1 if t % 2 else -1), int(r7.integers(-60, 61))]
        n = 3 * int(r7.integers(4, 900))
        tail = np.where(r7.random(n) < 0.5, 0, r7.integers(-80, 81, n))
        s = np.concatenate([head, tail])[:n]
        vecs.append(s.astype(np.int64))
        kinds.append(7)
    enc = [ref.rlgr_encode(v) for v in vecs]
    dec = [ref.rlgr_decode(e, v.size) for e, v in zip(enc, vecs)]
    off = np.cumsum([0] + [len(e) for e in enc])
    soff = np.cumsum([0] + [len(v) for v in vecs])
    np.savez_compressed(os.path.join(HERE, "rlgr.npz"), symbols=np.concatenate(vecs), sym_off=soff,
                        decoded=np.concatenate(dec), bytes=np.frombuffer(b"".join(enc), np.uint8), byte_off=off,
                        kinds=np.array(kinds))


def edge_patches(rng):
    """(xyz float32, rgb uint8) of the edge-case patches."""
    pats = []
    pats.append((np.array([[100.0, 200.0, 300.0]], np.float32), np.array([[10, 200, 30]], np.uint8)))
    pats.append((np.array([[0.0, 0.0, 0.0], [37.0, 5.0, 90.0]], np.float32), np.array([[0, 0, 0], [255, 255, 255]], np.uint8)))
    g = np.stack(np.meshgrid(np.arange(8), np.arange(8), np.arange(8), indexing="ij"), -1).reshape(-1, 3)
    pats.append(((g + 40).astype(np.float32), rng.integers(0, 256, (512, 3)).astype(np.uint8)))
    p = rng.integers(0, 20, (300, 3)).astype(np.float32) + np.float32(0.5)
    p = np.concatenate([p, p[:60]])                                     # shared voxels
    pats.append((p, rng.integers(30, 220, (p.shape[0], 3)).astype(np.uint8)))
    return pats


def make_gop_encode(ref: Reference, seed: int = 41):
    """Fitting clouds from the synthetic generator; each frame's source patch
    is the cloud moved by up to a voxel per axis with 10% of points dropped,
    integer coordinates (many equal distances), random RGB."""
    import pvvc
    s = pvvc.Synth(pvvc.config("gof8", nframes=3, gof=3, seed=seed))
    rng = np.random.default_rng(seed)
    out = {}
    fits, srcs, rgbs, cols, geos, pays = [], [], [], [], [], []
    for p in range(s.patch_count(0)):
        xyz = s.patch(0, p)[0].astype(np.float32)
        if xyz.shape[0] > 1200:
            continue
        ss, cc = [], []
        for f in range(3):
            keep = rng.random(xyz.shape[0]) > 0.1
            keep[0] = True
            ss.append(np.round(xyz[keep] + rng.integers(-1, 2, (int(keep.sum()), 3))).astype(np.float32))
            cc.append(rng.integers(0, 256, (int(keep.sum()), 3)).astype(np.uint8))
        c, g, pl = ref.gop_encode(xyz, ss, cc, 10, QP_I, QP_P)
        fits.append(xyz)
        srcs += ss
        rgbs += cc
        cols.append(c.reshape(-1, 3))
        geos.append(np.frombuffer(g, np.uint8))
        pays += [np.frombuffer(x, np.uint8) for x in pl]
        if len(fits) == 4:
            break
    cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0)
    off = lambda xs: np.concatenate([[0], np.cumsum([len(x) for x in xs])]).astype(np.int64)
    np.savez_compressed(os.path.join(HERE, "gop_encode.npz"), k=10, qp_i=QP_I, qp_p=QP_P, nframes=3,
                        fit=cat(fits), fit_off=off(fits), src=cat(srcs), src_off=off(srcs), rgb=cat(rgbs),
                        colors=cat(cols), geo=cat(geos), geo_off=off(geos), pay=cat(pays), pay_off=off(pays))


def make_cloud_mse(ref: Reference, seed: int = 43):
    """Voxel clouds against each other, and synthetic patches against a
    rotated, shifted and jittered copy (the registration's use)."""
    import pvvc
    rng = np.random.default_rng(seed)
    a_list, b_list = [], []
    for _ in range(3):
        a_list.append(rng.integers(0, 40, (int(rng.integers(50, 900)), 3)).astype(np.float32))
        b_list.append(rng.integers(0, 40, (int(rng.integers(50, 900)), 3)).astype(np.float32))
    s = pvvc.Synth(pvvc.config("gof8", nframes=1, gof=1, seed=seed))
    for p in range(3):
        x = s.patch(0, p)[0].astype(np.float32)
        R = rot(rng.normal(size=3), 5.0)
        y = ((x - x.mean(0)) @ R.T + x.mean(0) + rng.uniform(-2, 2, 3) + rng.normal(0, 0.5, x.shape)).astype(np.float32)
        a_list.append(x)
        b_list.append(y)
    mse = np.array([ref.cloud_mse(a, b) for a, b in zip(a_list, b_list)], np.float32)
    off = lambda xs: np.concatenate([[0], np.cumsum([len(x) for x in xs])]).astype(np.int64)
    np.savez_compressed(os.path.join(HERE, "cloud_mse.npz"), a=np.concatenate(a_list), a_off=off(a_list),
                        b=np.concatenate(b_list), b_off=off(b_list), mse=mse)


def make_cloud_quality(ref: Reference, seed: int = 47):
    """Coloured clouds: voxel clouds with many equidistant neighbours, and
    synthetic patches against a moved, jittered, recoloured copy (a decoded
    frame against its source)."""
    import pvvc
    rng = np.random.default_rng(seed)
    a_list, b_list, ac_list, bc_list = [], [], [], []
    for _ in range(3):
        a_list.append(rng.integers(0, 30, (int(rng.integers(50, 900)), 3)).astype(np.float32))
        b_list.append(rng.integers(0, 30, (int(rng.integers(50, 900)), 3)).astype(np.float32))
    s = pvvc.Synth(pvvc.config("gof8", nframes=1, gof=1, seed=seed))
    for p in range(3):
        x = s.patch(0, p)[0].astype(np.float32)
        R = rot(rng.normal(size=3), 1.0)
        y = ((x - x.mean(0)) @ R.T + x.mean(0) + rng.uniform(-1, 1, 3) + rng.normal(0, 0.3, x.shape)).astype(np.float32)
        a_list.append(x)
        b_list.append(np.round(y).astype(np.float32))
    for k, (a, b) in enumerate(zip(a_list, b_list)):
        ac_list.append(rng.integers(0, 256, a.shape).astype(np.uint8))
        if k < 3:  # unrelated colours
            bc_list.append(rng.integers(0, 256, b.shape).astype(np.uint8))
        else:      # the same points' colours with N(0, 6) noise
            bc_list.append(np.clip(np.round(ac_list[-1] + rng.normal(0, 6, b.shape)), 0, 255).astype(np.uint8))
    mse = np.array([ref.mse_compute(a, ac, b, bc) for a, ac, b, bc in zip(a_list, ac_list, b_list, bc_list)], np.float64)
    off = lambda xs: np.concatenate([[0], np.cumsum([len(x) for x in xs])]).astype(np.int64)
    np.savez_compressed(os.path.join(HERE, "cloud_quality.npz"), a=np.concatenate(a_list), a_rgb=np.concatenate(ac_list),
                        a_off=off(a_list), b=np.concatenate(b_list), b_rgb=np.concatenate(bc_list), b_off=off(b_list),
                        mse=mse)


def make_fitting(ref: Reference):
    """GoPs of registered patches -> the reference's fitting clouds."""
    import pvvc
    s = pvvc.Synth(pvvc.config("gof8", seed=21))
    cases = []  # (list of patches, seed)
    for p in range(3):
        xyz, yuv, mv = s.patch(0, p)
        rng = np.random.default_rng(100 + p)
        pats = [xyz.astype(np.float32)]
        for f in range(1, mv.shape[0]):
            # the frame's patch (moved, jittered, voxelised), registered back by the true motion
            m = mv[f].astype(np.float64)
            moved = np.round(xyz @ m[:3, :3].T + m[:3, 3] + rng.normal(0, 0.3, xyz.shape))
            inv = np.linalg.inv(m)
            pats.append((moved @ inv[:3, :3].T + inv[:3, 3]).astype(np.float32))
        cases.append((pats, 1 + p))
        cases.append((pats[:3], 7))
    rng = np.random.default_rng(0)
    for t in range(12):  # repeated points: empty clusters, redrawn from rand()
        base = rng.integers(0, 6, (int(rng.integers(4, 30)), 3)).astype(np.float32)
        pats = [base[rng.integers(0, base.shape[0], int(rng.integers(5, 40)))] for _ in range(int(rng.integers(3, 6)))]
        if t in (0, 2, 4):
            cases.append((pats, t))
    allp, poff, gop, seeds, outs, ooff = [], [0], [0], [], [], [0]
    for pats, seed in cases:
        for x in pats:
            allp.append(x)
            poff.append(poff[-1] + x.shape[0])
        gop.append(gop[-1] + len(pats))
        seeds.append(seed)
        y = ref.fitting_cloud(pats, seed=seed)
        outs.append(y)
        ooff.append(ooff[-1] + y.shape[0])
    np.savez_compressed(os.path.join(HERE, "fitting.npz"), xyz=np.concatenate(allp), patch_off=np.array(poff, np.int64),
                        gop_patch=np.array(gop, np.int64), seeds=np.array(seeds, np.uint32), fit=np.concatenate(outs),
                        fit_off=np.array(ooff, np.int64))


def main():
    ref = Reference()
    one = {"gop_encode": make_gop_encode, "cloud_mse": make_cloud_mse, "cloud_quality": make_cloud_quality,
           "fitting": make_fitting}
    if len(sys.argv) == 2 and sys.argv[1] in one:
        one[sys.argv[1]](ref)
        print(sys.argv[1] + ".npz written to", HERE)
        return
    make_gop_encode(ref)
    make_cloud_mse(ref)
    make_cloud_quality(ref)
    make_fitting(ref)
    rng = np.random.default_rng(2024)
    make_rlgr(ref, rng)

    import pvvc  # the synthetic surface generator (host C++), for realistic patches
    s = pvvc.Synth(pvvc.config("gof8", nframes=NFRAMES, gof=NFRAMES, seed=7))
    patches = []
    for p in range(4):
        xyz, yuv, mv = s.patch(0, p)
        patches.append(("synth", xyz, yuv, mv))
    for xyz, rgb in edge_patches(rng):
        yuv0 = rgb_to_yuv(rgb)
        yuv = [yuv0] + [rng.normal(0, 40, yuv0.shape).astype(np.float32) for _ in range(NFRAMES - 1)]
        mv = [np.eye(4, dtype=np.float32)]
        for f in range(1, NFRAMES):
            m = np.eye(4)
            m[:3, :3] = rot(rng.normal(size=3), 2.0 * f)
            m[:3, 3] = rng.uniform(-3, 3, 3)
            mv.append(m.astype(np.float32))
        patches.append(("edge", xyz, np.stack(yuv), np.stack(mv)))

    outdir = os.path.join(HERE, "gop")
    if os.path.isdir(outdir):
        shutil.rmtree(outdir)
    os.makedirs(outdir)
    expected = {}
    tmp = tempfile.mkdtemp()
    decs = [ref.decoder() for _ in patches]
    for variant in ("raw", "zstd"):
        for f in range(NFRAMES):
            d = os.path.join(tmp, f"{variant}_{f}")
            os.makedirs(d)
            for pi, (_, xyz, yuv, mv) in enumerate(patches):
                qp = QP_I if f == 0 else QP_P
                geo, nl, cols, _ = ref.encode_patch(xyz, [yuv[f]], [qp], quantise)
                col = cols[0]
                typ = 0x01 if f == 0 else 0x03
                if variant == "zstd":           # GoPEncoding: keep zstd only when it is smaller
                    if f == 0:
                        gz = ref.zstd_encode(geo, 22)
                        if len(gz) < len(geo):
                            geo, typ = gz, typ | 0x08
                    cz = ref.zstd_encode(col, 22)
                    if len(cz) < len(col):
                        col, typ = cz, typ | 0x10
                mv_cm = mv[f].T.reshape(16).astype(np.float32)   # Slice.mv is column-major
                name = os.path.join(d, f"golden_time_{f:04d}_slice_{pi:04d}.slice")
                u8 = ctypes.POINTER(ctypes.c_uint8)
                gbuf = np.frombuffer(geo, np.uint8).copy()
                cbuf = np.frombuffer(col, np.uint8).copy()
                rc = ref.lib.ref_save_slice(name.encode(), typ, f, pi, nl, qp, mv_cm.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                            gbuf.ctypes.data_as(u8) if f == 0 else None, len(geo) if f == 0 else 0,
                                            cbuf.ctypes.data_as(u8), len(col))
                assert rc > 0, rc
                if variant == "raw":
                    dec = decs[pi]
                    assert dec.set_slice(typ, nl, qp, geo if f == 0 else b"", col, mv_cm, f, pi) == 0
                    pxyz, prgb = dec.get_patch(nl)
                    expected.setdefault(f"xyz_{f}", []).append(transform(pxyz, mv[f]))
                    expected.setdefault(f"rgb_{f}", []).append(prgb)
            out = os.path.join(outdir, f"{variant}_{f}.frame")
            assert ref.lib.ref_change_slice_to_frame(d.encode(), out.encode()) == 0
    shutil.rmtree(tmp)
    np.savez_compressed(os.path.join(outdir, "expected.npz"), **{k: np.concatenate(v) for k, v in expected.items()})
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
