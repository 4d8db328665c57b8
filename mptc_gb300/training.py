"""Training of the learned proposal on seeded frames.

The plain (exhaustive, bit-exact) GPU encoder labels every inter-frame block
with the candidate the reference's search accepts. A training example is that
(block, accepted candidate) pair plus C-1 other distinct index words of the
block's window that the exhaustive search rates strictly worse (a higher
err_diff, or a refit that would swap the endpoints), their exact err_diff
computed on the GPU by mptc_candidate_errors; words as good as the accepted
one are never used as negatives. Steps run in the library's kernels (sampled
softmax cross-entropy, AdamW).
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
from numpy.lib.stride_tricks import sliding_window_view

from ._lib import check, dev_ptr, lib
from .encoder import Encoder, intra_schedule
from .model import ProposalModel

INVALID = 0x7FFFFFFF  # err_diff of a candidate whose refit would swap the endpoints


def window_words(prev_final: np.ndarray, bw: int, bh: int, sa: int) -> np.ndarray:
    """(bh*bw, (2sa)^2) index words of every block's inter window in the
    reference's scan order (rows by-sa.., columns bx-sa..), -1 outside the frame."""
    prev = (prev_final >> np.uint64(32)).astype(np.int64).reshape(bh, bw)
    pad = np.full((bh + 2 * sa, bw + 2 * sa), -1, np.int64)
    pad[sa:sa + bh, sa:sa + bw] = prev
    return sliding_window_view(pad, (2 * sa, 2 * sa))[:bh, :bw].reshape(bh * bw, 4 * sa * sa)


def accepted_inter(motion: np.ndarray, bw: int, sa: int):
    """Blocks the search accepted with an inter match and their window position."""
    m = motion.reshape(-1, 2).astype(np.int64)
    inter = np.nonzero((m[:, 0] >= 128) & ~((m[:, 0] == 255) & (m[:, 1] == 255)))[0]
    pos = (m[inter, 1] - 128) * (2 * sa) + (m[inter, 0] - 128)
    return inter, pos


def distinct_words(win: np.ndarray, exclude: np.ndarray, rng: np.random.Generator, k: int):
    """Up to k distinct in-frame words of each row other than exclude[row], in
    random order; (words (rows, k) with -1 padding, counts)."""
    w = win.copy()
    w[w == exclude[:, None]] = -1
    s = np.sort(w, axis=1)
    first = np.ones_like(s, dtype=bool)
    first[:, 1:] = s[:, 1:] != s[:, :-1]
    first &= s >= 0
    key = np.where(first, rng.random(s.shape), 2.0)
    order = np.argsort(key, axis=1)[:, :k]
    out = np.take_along_axis(s, order, 1)
    ok = np.take_along_axis(first, order, 1)
    return np.where(ok, out, -1), ok.sum(1)


def candidate_errors(torch, rgb, width, height, stb, blocks, cands) -> np.ndarray:
    """Exact err_diff of cands (B x C words) on blocks of a frame (device tensors)."""
    B, C = cands.shape
    err = torch.empty((B, C), dtype=torch.int32, device=rgb.device)
    check(lib().mptc_candidate_errors(dev_ptr(rgb, "rgb", 1, width * height * 3), width, height,
                                      dev_ptr(stb, "stb", 8, (width // 4) * (height // 4)),
                                      dev_ptr(blocks, "blocks", 4, B), dev_ptr(cands, "cands", 4, B * C), B, C,
                                      dev_ptr(err, "err", 4, B * C), ctypes.c_void_p(0)))
    return err.cpu().numpy()


def frame_examples(torch, rgb, width, height, stb, motion, prev_final, sa, rng, per_frame, cands, pool=48):
    """Training examples of one inter frame: (blocks int32 (B,), cands uint32 (B, C))
    with the accepted word first, or None."""
    bw, bh = width // 4, height // 4
    inter, pos = accepted_inter(motion, bw, sa)
    if inter.size == 0:
        return None
    pick = rng.choice(inter.size, min(per_frame, inter.size), replace=False)
    blocks, pos = inter[pick], pos[pick]
    win = window_words(prev_final, bw, bh, sa)[blocks]
    acc = win[np.arange(blocks.size), pos]
    others, _ = distinct_words(win, acc, rng, pool)
    # label the accepted word and the pool with the exhaustive search's err_diff
    lab = np.concatenate([acc[:, None], np.where(others >= 0, others, acc[:, None])], 1).astype(np.uint32)
    dev = rgb.device
    err = candidate_errors(torch, rgb, width, height, stb, torch.from_numpy(blocks.astype(np.int32)).to(dev),
                           torch.from_numpy(lab.view(np.int32)).to(dev))
    worse = (others >= 0) & (err[:, 1:].astype(np.int64) > err[:, :1].astype(np.int64))
    n_neg = worse.sum(1)
    keep = n_neg > 0
    if not keep.any():
        return None
    # negatives: the strictly worse words, cycled to fill C-1 slots
    order = np.argsort(~worse, axis=1, kind="stable")
    neg = np.take_along_axis(others, order, 1)
    slot = np.arange(cands - 1)[None, :] % np.maximum(n_neg, 1)[:, None]
    neg = np.take_along_axis(neg, slot, 1)
    out = np.concatenate([acc[:, None], neg], 1)[keep].astype(np.uint32)
    return blocks[keep].astype(np.int32), out


def train_proposal(torch, frames_dev, search_area=8, err_threshold=5, intra_interval=16, steps=2000,
                   batch=4096, cands=32, lr=1e-3, weight_decay=1e-4, seed=0, per_frame=4096, log=None):
    """frames_dev: (T, H, W, 3) uint8 CUDA tensor. Returns (model, losses, info)."""
    T, H, W, _ = frames_dev.shape
    n = (W // 4) * (H // 4)
    dev = frames_dev.device
    t0 = time.time()
    enc = Encoder(W, H, search_area, err_threshold, intra_interval)
    flags = intra_schedule(T, intra_interval)
    fin = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(2)]
    mot = torch.empty(2 * n, dtype=torch.uint8, device=dev)
    uni = torch.empty(n, dtype=torch.int32, device=dev)
    nu = torch.zeros(1, dtype=torch.int32, device=dev)
    rng = np.random.default_rng(seed)
    stbs, examples = [], []
    prev_host = None
    for t in range(T):
        stb = torch.empty(n, dtype=torch.int64, device=dev)
        prev = None if flags[t] else fin[(t - 1) % 2]
        enc.encode_frame_device(frames_dev[t], prev, stb, fin[t % 2], mot, uni, nu)
        fin_host = fin[t % 2].cpu().numpy().view(np.uint64).copy()
        stbs.append(stb)
        if not flags[t] and prev_host is not None:
            ex = frame_examples(torch, frames_dev[t], W, H, stb, mot.cpu().numpy(), prev_host, search_area, rng,
                                per_frame, cands)
            if ex is not None:
                examples.append((t, torch.from_numpy(ex[0]).to(dev), torch.from_numpy(ex[1].view(np.int32)).to(dev)))
        prev_host = fin_host
    enc.close()
    label_s = time.time() - t0
    model = ProposalModel(seed=seed)
    losses = []
    t1 = time.time()
    for s in range(steps):
        t, blocks, cnd = examples[int(rng.integers(len(examples)))]
        if blocks.numel() > batch:
            sel = torch.from_numpy(rng.choice(blocks.numel(), batch, replace=False)).to(dev)
            blocks, cnd = blocks[sel], cnd[sel]
        losses.append(model.train_step(frames_dev[t], W, stbs[t], blocks.contiguous(), cnd.contiguous(), lr=lr,
                                       weight_decay=weight_decay))
        if log is not None and (s % 250 == 0 or s == steps - 1):
            log(f"train step {s}: loss {losses[-1]:.4f}")
    torch.cuda.synchronize()
    info = dict(frames=T, examples=int(sum(e[1].numel() for e in examples)), label_seconds=round(label_s, 2),
                train_seconds=round(time.time() - t1, 2), steps=steps, batch=batch, candidates=cands)
    return model, losses, info


def decoded_sse(torch, rgb, width, height, blocks) -> int:
    """Squared error of a frame against its decoded DXT1 blocks (device tensors)."""
    sse = torch.zeros(1, dtype=torch.int64, device=rgb.device)
    check(lib().mptc_decoded_sse(dev_ptr(rgb, "rgb", 1, width * height * 3), width, height,
                                 dev_ptr(blocks, "blocks", 8, (width // 4) * (height // 4)),
                                 dev_ptr(sse, "sse", 8, 1), ctypes.c_void_p(0)))
    return int(sse.item())


def choose_topk(torch, model, frames_dev, search_area=8, err_threshold=5, intra_interval=16, ks=(4, 8, 16),
                max_psnr_loss_db=0.05, log=None):
    """The number of proposals per block, chosen against the exhaustive search:
    the calibration frames are encoded by the exhaustive search and with each
    K; the fastest K whose decoded PSNR stays within max_psnr_loss_db of the
    exhaustive search's is kept (half the 0.1 dB budget, the rest is margin
    for content the calibration frames do not show), else the most accurate.
    Returns (K, {K: (psnr loss dB, ms per frame, fallback rate)})."""
    T, H, W, _ = frames_dev.shape
    n = (W // 4) * (H // 4)
    dev = frames_dev.device
    flags = intra_schedule(T, intra_interval)
    s = torch.cuda.current_stream()

    def run(K):
        enc = Encoder(W, H, search_area, err_threshold, intra_interval)
        if K:
            enc.set_model(model, K)
        fin = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(2)]
        mot = torch.empty(2 * n, dtype=torch.uint8, device=dev)
        uni = torch.empty(n, dtype=torch.int32, device=dev)
        nu = torch.zeros(1, dtype=torch.int32, device=dev)
        sse, fb, inter, ms = 0, 0, 0, 0.0
        for rep in range(2):  # the second pass is timed
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for t in range(T):
                prev = None if flags[t] else fin[(t - 1) % 2]
                enc.encode_frame_device(frames_dev[t], prev, None, fin[t % 2], mot, uni, nu, s)
                if rep == 1:
                    sse += decoded_sse(torch, frames_dev[t], W, H, fin[t % 2])
                    if not flags[t]:
                        fb += enc.stats(s).n_fallback
                        inter += n
            e1.record(s)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / T
        enc.close()
        return sse, ms, fb / max(1, inter)

    base_sse, base_ms, _ = run(0)
    table = {}
    for K in ks:
        sse, ms, fb = run(K)
        loss = 10.0 * float(np.log10(max(sse, 1) / max(base_sse, 1)))
        table[K] = (round(loss, 4), round(ms, 3), round(fb, 4))
        if log is not None:
            log(f"K={K}: PSNR loss {loss:.4f} dB, {ms:.3f} ms/frame (exhaustive {base_ms:.3f}), fallback {fb:.4f}")
    ok = [K for K in ks if table[K][0] <= max_psnr_loss_db]
    best = min(ok, key=lambda K: table[K][1]) if ok else min(ks, key=lambda K: table[K][0])
    return best, table


def main(argv=None) -> None:
    """Trains the proposal on the seeded 1080p training frames and prints the
    labelling and training times (ms per AdamW step) as one JSON line;
    --out writes the weights (ProposalModel.load reads them back)."""
    import argparse
    import json

    import torch

    from .synth import FHD1080_TRAIN
    ap = argparse.ArgumentParser(prog="python -m mptc_gb300.training")
    ap.add_argument("--frames", type=int, default=FHD1080_TRAIN.frames, help="training frames (a prefix of the 200)")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--cands", type=int, default=32)
    ap.add_argument("--out", default="")
    args = ap.parse_args(argv)
    frames = torch.from_numpy(FHD1080_TRAIN.generate(0, args.frames)).cuda()
    model, losses, info = train_proposal(torch, frames, steps=args.steps, batch=args.batch, cands=args.cands)
    info.update(ms_per_step=round(1e3 * info["train_seconds"] / max(1, args.steps), 3),
                first_loss=round(losses[0], 4), last_loss=round(losses[-1], 4))
    if args.out:
        model.save(args.out)
    model.close()
    print(json.dumps(info), flush=True)


if __name__ == "__main__":
    main()
