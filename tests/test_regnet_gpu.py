"""The registration network on the GPU (regnet.cu + the tcgen05 GEMM):
gradients against the CPU oracle (oracle/regnet_oracle.py), a training run
on ICP-labelled synthetic pairs, and what the trained proposer gains over
plain ICP from the identity.

Gradient tolerance: per parameter block, |g_gpu - g_oracle| <= 2e-2 |g_oracle|
(Frobenius).  Both sides round to bf16 at the same points; what remains is
fp32 reassociation in the GEMMs and the occasional bf16 rounding flip it
causes.  Loss: relative 1e-3."""
import numpy as np
import pytest

import regnet_oracle as ro

pytestmark = pytest.mark.gpu

GRAD_RTOL = 2e-2


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def _blocks(a):
    out, o = {}, 0
    for k, s in ro.DIMS.items():
        n = int(np.prod(s))
        out[k] = a[o:o + n]
        o += n
    return out


@pytest.mark.parametrize("B,seed", [(64, 0), (128, 1)])
def test_gradient_matches_oracle(pvvc_lib, torch, B, seed):
    from pvvc.regnet import RegNet
    net = RegNet(seed=seed)
    flat = net.get_params()
    rng = np.random.default_rng(100 + seed)
    x0 = rng.normal(0, 1, (B, 2, ro.P, 3)).astype(np.float32)
    y = rng.normal(0, 0.5, (B, 6)).astype(np.float32)
    g, loss = net.grad(torch.from_numpy(x0).cuda(), torch.from_numpy(y).cuda(), 4.0,
                       stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    lref, gref, _ = ro.loss_and_grad(flat, x0, y, 4.0)
    assert abs(float(loss.item()) - lref) <= 1e-3 * abs(lref)
    gg, gr = _blocks(g.cpu().numpy()), _blocks(gref)
    for k in ro.DIMS:
        err = np.linalg.norm(gg[k] - gr[k])
        assert err <= GRAD_RTOL * np.linalg.norm(gr[k]) + 1e-7, (k, err, np.linalg.norm(gr[k]))


def test_params_round_trip_and_reset(pvvc_lib, torch):
    from pvvc.regnet import RegNet
    a, b = RegNet(seed=5), RegNet(seed=6)
    pa = a.get_params()
    assert not np.array_equal(pa, b.get_params())
    b.set_params(pa)
    assert np.array_equal(b.get_params(), pa)
    assert pa.size == pvvc_lib.lib().pvvc_regnet_param_count()


def _labelled(pvvc_lib, torch, n, seed, synth_seed):
    from pvvc.icp import IcpBatch, make_pairs
    from pvvc.regnet import PairData
    s = pvvc_lib.Synth(pvvc_lib.config("seq300", nframes=1, gof=1, seed=synth_seed))
    pairs = make_pairs(n, seed=seed, synth=s)
    b = IcpBatch(pairs)
    b.run(max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
    T, mse, _, _ = b.results()
    return pairs, b, PairData(b, T), mse


@pytest.fixture(scope="module")
def trained(pvvc_lib, torch):
    """A network trained for 600 steps (batch 256) on 2048 ICP-labelled pairs
    of one synthetic surface, with its loss curve."""
    from pvvc.regnet import AdamW, RegNet
    _, _, train, _ = _labelled(pvvc_lib, torch, 2048, seed=11, synth_seed=21)
    net = RegNet(seed=0)
    opt = AdamW(1e-3, 0.9, 0.999, 1e-8, 1e-4, 4.0)
    g = torch.Generator(device="cpu").manual_seed(0)
    loss = torch.zeros(1, device="cuda")
    losses = []
    sp = torch.cuda.current_stream().cuda_stream
    for it in range(600):
        ids = torch.randint(0, train.n, (256,), generator=g, dtype=torch.int32).cuda()
        net.train_step(train, ids, seed=it, opt=opt, loss_out=loss, stream=sp)
        if it % 50 == 0 or it == 599:
            losses.append(float(loss.item()))
    import ctypes
    c = ctypes.c_int32(-1)
    assert pvvc_lib.lib().pvvc_device_error_take(ctypes.byref(c)) == 0 and c.value == 0
    return net, losses


def test_training_reduces_loss(trained):
    _, losses = trained
    assert np.isfinite(losses).all()
    assert np.mean(losses[-3:]) < 0.3 * losses[0], losses


def test_proposals_beat_identity_at_equal_iterations(pvvc_lib, torch, trained):
    """On 512 pairs of another surface, 10 ICP iterations from the proposals
    leave a lower registration MSE than 10 from the identity."""
    net, _ = trained
    _, b, test, _ = _labelled(pvvc_lib, torch, 512, seed=12, synth_seed=22)
    T0 = net.propose(test, seed=1, stream=torch.cuda.current_stream().cuda_stream)
    b.run(init=T0, max_iter=10, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
    _, learned10, _, _ = b.results()
    b.run(max_iter=10, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)
    _, plain10, _, _ = b.results()
    assert learned10.mean() < plain10.mean(), (learned10.mean(), plain10.mean())


def test_register_learned_is_no_worse_than_plain(pvvc_lib, torch, trained):
    """register_learned: with the plain-ICP judge every pair's MSE is at most
    plain ICP's; with the convergence judge (refinement converged, else plain
    ICP from the identity) the mean MSE stays within 2% of plain ICP's and
    the pairs handed to the fallback get exactly the plain result."""
    from pvvc.regnet import register_learned
    net, _ = trained
    _, b, _, plain50 = _labelled(pvvc_lib, torch, 512, seed=13, synth_seed=23)
    Tp = b.T.clone()
    _, mse_j, info_j = register_learned(net, b, judge="plain", plain=(Tp, torch.from_numpy(plain50).cuda()))
    mj = mse_j.cpu().numpy()
    assert (mj <= plain50).all()
    T_c, mse_c, info_c = register_learned(net, b, judge="converged")
    mc = mse_c.cpu().numpy()
    fb = ~info_c["accepted"].cpu().numpy()
    assert int(fb.sum()) == info_c["fallback"]
    assert np.allclose(mc[fb], plain50[fb], rtol=1e-6, atol=0)
    assert mc.mean() <= 1.02 * plain50.mean(), (mc.mean(), plain50.mean(), info_c)
