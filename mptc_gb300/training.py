"""Training loop of the learned proposal on seeded frames.

The plain (exhaustive, bit-exact) GPU encoder labels every inter-frame block
with the candidate the reference's search accepts; each training example is
that (block, accepted candidate) pair plus C-1 other candidates from the same
block's window. Steps run in the library's tensor-core kernels with AdamW.
"""
from __future__ import annotations

import numpy as np

from .encoder import Encoder, intra_schedule
from .model import ProposalModel, sample_examples


def train_proposal(torch, frames_dev, search_area=8, err_threshold=5, intra_interval=16, steps=400,
                   batch=4096, cands=16, lr=1e-3, weight_decay=1e-4, seed=0, log=None):
    """frames_dev: (T, H, W, 3) uint8 CUDA tensor. Returns (model, losses)."""
    T, H, W, _ = frames_dev.shape
    bw, bh = W // 4, H // 4
    n = bw * bh
    dev = frames_dev.device
    enc = Encoder(W, H, search_area, err_threshold, intra_interval)
    flags = intra_schedule(T, intra_interval)
    fin = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(2)]
    mot = torch.empty(2 * n, dtype=torch.uint8, device=dev)
    uni = torch.empty(n, dtype=torch.int32, device=dev)
    nu = torch.zeros(1, dtype=torch.int32, device=dev)
    stbs, examples = [], []
    rng = np.random.default_rng(seed)
    prev_final_host = None
    for t in range(T):
        stb = torch.empty(n, dtype=torch.int64, device=dev)
        prev = None if flags[t] else fin[(t - 1) % 2]
        enc.encode_frame_device(frames_dev[t], prev, stb, fin[t % 2], mot, uni, nu)
        final_host = fin[t % 2].cpu().numpy().view(np.uint64)
        stbs.append(stb)
        ex = None
        if not flags[t] and prev_final_host is not None:
            ex = sample_examples(rng, bw, bh, search_area, mot.cpu().numpy(), prev_final_host, batch, cands)
        if ex is not None:
            examples.append((t, torch.from_numpy(ex.blocks).to(dev), torch.from_numpy(ex.cands.view(np.int32)).to(dev)))
        prev_final_host = final_host
    enc.close()
    model = ProposalModel(seed=seed)
    losses = []
    for s in range(steps):
        t, blocks, cnd = examples[s % len(examples)]
        losses.append(model.train_step(frames_dev[t], W, stbs[t], blocks, cnd, lr=lr, weight_decay=weight_decay))
        if log is not None and (s % 100 == 0 or s == steps - 1):
            log(f"train step {s}: loss {losses[-1]:.4f}")
    return model, losses
