"""Training of the patch-registration network on the GPU.

    python -m pvvc.train_regnet --pairs 200000 --epochs 20 --batch 1024 --out regnet.npz

Data: seeded synthetic patch pairs (make_pairs_packed: a patch of a
synthetic surface, its target rotated 0-15 deg about a uniform axis through
the centroid, translated within +-20 voxels, N(0, 0.5) jitter, 5% outliers),
from several surfaces, generated on the device in chunks.  Labels: the
transform plain GPU ICP converges to from the identity (pvvc_icp_batch, 50
iterations), as the encoder would compute it.  Training: pvvc_regnet_train_step
(sampling, tcgen05 forward and backward, AdamW) with a cosine learning rate.
Output: an .npz with the flat fp32 parameters (`params`) and the loss curve."""
from __future__ import annotations

import argparse
import math
import time

import numpy as np

ICP = dict(max_corr_dist=1e6, max_iter=50, fitness_eps=0.0, transform_eps=0.0, mse_abs_eps=1e-6)


def labelled_dataset(npairs: int, seed: int, surfaces: int = 4, chunk: int = 16384, log=print):
    """Device-resident pairs with ICP labels, from `surfaces` synthetic
    surfaces (seeds seed .. seed+surfaces-1)."""
    import torch

    from .icp import IcpBatch, make_pairs_packed
    from .regnet import PairData
    from .synth import Synth, config
    synths = [Synth(config("seq300", nframes=1, gof=1, seed=seed + i)) for i in range(surfaces)]
    parts, Ts, mses = [], [], []
    done = 0
    t0 = time.time()
    while done < npairs:
        n = min(chunk, npairs - done)
        k = len(parts)
        src, so, tgt, to, _ = make_pairs_packed(n, seed=seed * 1000 + k, synth=synths[k % surfaces])
        b = IcpBatch(None, packed=(src, so, tgt, to))
        b.run(**ICP)
        T, mse, _, _ = b.results()
        parts.append((src, so, tgt, to))
        Ts.append(T)
        mses.append(mse)
        done += n
        del b
    src = torch.cat([p[0] for p in parts])
    tgt = torch.cat([p[2] for p in parts])
    sb = np.cumsum([0] + [int(p[0].shape[0]) for p in parts])
    tb = np.cumsum([0] + [int(p[2].shape[0]) for p in parts])
    so = torch.cat([parts[0][1][:1]] + [p[1][1:] + int(sb[i]) for i, p in enumerate(parts)])
    to = torch.cat([parts[0][3][:1]] + [p[3][1:] + int(tb[i]) for i, p in enumerate(parts)])
    data = PairData.from_packed(src, so, tgt, to, np.concatenate(Ts))
    log(f"dataset: {npairs} pairs, {int(so[-1])} + {int(to[-1])} points, ICP-labelled in {time.time() - t0:.1f}s, "
        f"mean label MSE {float(np.concatenate(mses).mean()):.3f}")
    return data


def train(net, data, epochs: int, batch: int, lr: float, weight_decay: float = 1e-4, lambda_w: float = 4.0,
          seed: int = 0, log=print, log_every: int = 100):
    """AdamW with a cosine schedule from lr to 0 over all steps.  Returns the
    loss of every step (numpy)."""
    import torch

    from .regnet import AdamW
    steps_per_epoch = data.n // batch
    total = epochs * steps_per_epoch
    g = torch.Generator(device="cuda").manual_seed(seed)
    losses = torch.zeros(total, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    t0 = time.time()
    step = 0
    for ep in range(epochs):
        perm = torch.randperm(data.n, generator=g, device="cuda").to(torch.int32)
        for i in range(steps_per_epoch):
            ids = perm[i * batch:(i + 1) * batch]
            opt = AdamW(lr * 0.5 * (1 + math.cos(math.pi * step / total)), 0.9, 0.999, 1e-8, weight_decay, lambda_w)
            net.train_step(data, ids, seed=seed * 1_000_003 + step, opt=opt, loss_out=losses[step:step + 1], stream=sp)
            step += 1
            if log_every and step % log_every == 0:
                log(f"step {step}/{total} loss {float(losses[step - 1].item()):.4f} ({time.time() - t0:.1f}s)")
    torch.cuda.synchronize()
    return losses.cpu().numpy(), time.time() - t0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=200_000)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default="regnet.npz")
    a = ap.parse_args()
    from .regnet import RegNet
    data = labelled_dataset(a.pairs, seed=100 + a.seed)
    net = RegNet(seed=a.seed)
    losses, secs = train(net, data, a.epochs, a.batch, a.lr, seed=a.seed)
    np.savez(a.out, params=net.get_params(), losses=losses, pairs=a.pairs, epochs=a.epochs, batch=a.batch, lr=a.lr,
             train_seconds=secs)
    print(f"trained {len(losses)} steps in {secs:.1f}s; loss {losses[:10].mean():.4f} -> {losses[-10:].mean():.4f}; "
          f"saved {a.out}")


if __name__ == "__main__":
    main()
