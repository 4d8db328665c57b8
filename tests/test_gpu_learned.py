"""Learned candidate proposal: the tensor-core embedding kernels and the window
scoring against CPU references, the training kernels' gradients against a CPU
reference (torch fp32 with the BF16 operand rounding emulated) under per-layer
bounds derived from BF16 rounding, training progress and checkpoints, what a
trained network gains over an untrained one on held-out frames, the exact
candidate errors against the oracle, and the validity of a stream encoded with
the proposal (every accepted block satisfies the reference's acceptance rule,
the stream decodes back bit-exactly)."""
import ctypes
import os
import tempfile

import numpy as np
import pytest

from mptc_gb300.synth import StreamSpec

pytestmark = pytest.mark.gpu

# BF16 keeps 8 significant bits: one rounding moves a value by at most 2^-9 of
# it. The kernels round operands and activations to BF16 at the points the
# reference below emulates, so what remains is the FP32 accumulation order and
# the rounding of the few values that land on the other side of a BF16
# rounding boundary. Embeddings: |gpu - ref| <= 2^-6 * (|x| . |W| summed
# magnitude of the last layer) elementwise. Gradients: every layer's output
# gradient is rounded to BF16 on the GPU before each product (not in the
# reference), and the error of a backpropagated gradient is bounded by the
# magnitudes it was summed from, not by its (possibly cancelled) value: with
# M_L = |dz_L| at the top and M_l = (M_{l+1} |W_{l+1}|^T) * relu'(z_l) below,
# |gpu - ref| <= 2^-5 * (|h_{l-1}|^T M_l) elementwise for weights and
# 2^-5 * sum_rows M_l for biases.
EMB_TOL, GRAD_TOL = 2.0 ** -6, 2.0 ** -5


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def bf(torch, t):
    return t.to(torch.bfloat16).to(torch.float32)


def block_features(frame, stb, blocks, bw):
    """The 54 block features (zero padded to 64): pixel channels normalised to
    the block's own channel range, stb endpoints as 5/6/5-bit fractions."""
    X = np.zeros((len(blocks), 64), np.float32)
    for r, idx in enumerate(blocks):
        by, bx = divmod(int(idx), bw)
        px = frame[4 * by:4 * by + 4, 4 * bx:4 * bx + 4].reshape(16, 3).astype(np.float32)
        lo, hi = px.min(0), px.max(0)
        inv = np.where(hi > lo, np.float32(1.0) / np.maximum(hi - lo, 1).astype(np.float32), np.float32(0.0))
        X[r, :48] = ((px - lo) * inv).reshape(48)
        for k, ep in enumerate([int(stb[idx]) & 0xFFFF, (int(stb[idx]) >> 16) & 0xFFFF]):
            X[r, 48 + 3 * k:51 + 3 * k] = [(ep >> 11) / 31.0, ((ep >> 5) & 63) / 63.0, (ep & 31) / 31.0]
    return X


def cand_features(words):
    w = np.asarray(words, np.uint64).reshape(-1)
    return ((w[:, None] >> np.arange(32, dtype=np.uint64)[None, :]) & np.uint64(1)).astype(np.float32)


def layers(torch, params):
    from mptc_gb300.model import param_slices
    sl, _ = param_slices()
    p = torch.tensor(params, dtype=torch.float32, requires_grad=True)
    return p, [(p[a:b].view(*shp), p[c:d]) for (a, b, shp), (c, d, _) in sl]


def mlp(torch, Ws, x, ids):
    """Forward with BF16-rounded operands; returns (output, [(input, pre-activation) per layer])."""
    trace = []
    h = x
    for i, li in enumerate(ids):
        inp = bf(torch, h)
        z = inp @ bf(torch, Ws[li][0]) + Ws[li][1]
        if z.requires_grad:
            z.retain_grad()
        trace.append((inp, z))
        h = torch.relu(z) if i < len(ids) - 1 else z
    return h, trace


def make_batch(torch, w=128, h=64, B=48, C=8, seed=5):
    from mptc_gb300.encoder import Encoder
    frames = StreamSpec(w, h, 2, seed=seed).generate()
    enc = Encoder(w, h, 4, 5, 16)
    o0 = enc.encode_frame_host(frames[0], want_stb=True)
    o1 = enc.encode_frame_host(frames[1], want_stb=True)
    enc.close()
    rng = np.random.default_rng(seed)
    bw = w // 4
    blocks = rng.choice((w // 4) * (h // 4), B, replace=False).astype(np.int32)
    words = (o0.final >> np.uint64(32)).astype(np.uint32)
    cands = words[rng.integers(0, words.size, (B, C))]
    dev = torch.device("cuda")
    return dict(frame=frames[1], stb=o1.stb, blocks=blocks, cands=cands, bw=bw, w=w, prev=o0.final,
                rgb_d=torch.from_numpy(frames[1].copy()).to(dev),
                stb_d=torch.from_numpy(o1.stb.view(np.int64)).to(dev),
                blocks_d=torch.from_numpy(blocks).to(dev),
                cands_d=torch.from_numpy(cands.view(np.int32)).to(dev))


def test_embeddings_match_cpu_reference(torch_cuda):
    """The tcgen05 embedding kernels (through mptc_model_embed) against the
    CPU forward, elementwise, for a block list and for index words."""
    torch = torch_cuda
    from mptc_gb300.model import ProposalModel
    b = make_batch(torch, w=256, h=128, B=300, C=2)
    m = ProposalModel(seed=4)
    B = b["blocks"].size
    F = torch.empty((B, 64), dtype=torch.float32, device="cuda")
    G = torch.empty((B, 64), dtype=torch.float32, device="cuda")
    words = b["cands_d"][:, 0].contiguous()
    m.embed(b["rgb_d"], b["w"], b["stb_d"], b["blocks_d"], B, F, words, 1, B, G)
    torch.cuda.synchronize()
    _, Ws = layers(torch, m.params())
    with torch.no_grad():
        for got, x, ids in ((F, block_features(b["frame"], b["stb"], b["blocks"], b["bw"]), [0, 1, 2]),
                            (G, cand_features(b["cands"][:, 0]), [3, 4])):
            ref, trace = mlp(torch, Ws, torch.tensor(x), ids)
            inp, _ = trace[-1]
            mag = inp.abs() @ bf(torch, Ws[ids[-1]][0]).abs() + Ws[ids[-1]][1].abs()
            ref_b = bf(torch, ref)  # the kernels write bf16
            err = (got.cpu() - ref_b).abs()
            bound = EMB_TOL * mag + 2.0 ** -8 * ref.abs()
            assert bool((err <= bound).all()), float((err / bound).max())
    m.close()


@pytest.mark.parametrize("content", ["stream", "noise"])
def test_proposals_are_the_top_scored_distinct_words(torch_cuda, content):
    """mptc_learned_proposals against scores recomputed on the CPU from the
    same embeddings: in-frame window positions, K distinct words, each at its
    first position in scan order, and no word left out that scores clearly
    above the lowest one kept (the approximate top-K of an FP32 dot product).
    The stream frames' final blocks repeat dictionary words (a tile's word
    palette fits one slice); the noise frames' words are nearly all distinct,
    so a tile's palette spans several slices of 128 and of 64 entries."""
    torch = torch_cuda
    from mptc_gb300._lib import check, lib
    from mptc_gb300.encoder import Encoder
    from mptc_gb300.model import ProposalModel
    from mptc_gb300.training import window_words
    w, h, sa, K = 256, 192, 8, 8
    if content == "stream":
        frames = StreamSpec(w, h, 2, seed=21, n_squares=2, square_size=48).generate()
    else:
        frames = np.random.default_rng(22).integers(0, 256, size=(2, h, w, 3), dtype=np.uint8)
    bw, bh = w // 4, h // 4
    n = bw * bh
    enc = Encoder(w, h, sa, 5, 16)
    o0 = enc.encode_frame_host(frames[0], want_stb=True)
    o1 = enc.encode_frame_host(frames[1], want_stb=True)
    m = ProposalModel(seed=11)
    enc.set_model(m, K)
    dev = torch.device("cuda")
    rgb = torch.from_numpy(frames[1].copy()).to(dev)
    stb = torch.from_numpy(o1.stb.view(np.int64).copy()).to(dev)
    prev = torch.from_numpy(o0.final.view(np.int64).copy()).to(dev)
    for rows in (8, 4):
        check(lib().mptc_ctx_set_learned_shape(enc.handle, rows))
        topk = torch.empty((n, 16), dtype=torch.int16, device=dev)
        check(lib().mptc_learned_proposals(enc.handle, rgb.data_ptr(), stb.data_ptr(), prev.data_ptr(),
                                           topk.data_ptr(), ctypes.c_void_p(0)), enc.handle)
        tk = topk.cpu().numpy().view(np.uint16).astype(np.int64)
        F = torch.empty((n, 64), dtype=torch.float32, device=dev)
        G = torch.empty((n, 64), dtype=torch.float32, device=dev)
        words_d = torch.from_numpy((o0.final >> np.uint64(32)).astype(np.uint32).view(np.int32)).to(dev)
        m.embed(rgb, w, stb, None, n, F, words_d, 1, n, G)
        Fh, Gh = F.cpu().numpy().astype(np.float64), G.cpu().numpy().astype(np.float64)
        win = window_words(o0.final, bw, bh, sa)
        ys, xs = np.divmod(np.arange(n), bw)
        w2 = 2 * sa
        gy = ys[:, None] - sa + np.arange(w2 * w2)[None, :] // w2
        gx = xs[:, None] - sa + np.arange(w2 * w2)[None, :] % w2
        inside = (gy >= 0) & (gy < bh) & (gx >= 0) & (gx < bw)
        S = np.einsum("nd,npd->np", Fh, Gh[np.clip(gy * bw + gx, 0, n - 1)])
        tol = 1e-4 * np.abs(S[inside]).max()
        for idx in range(n):
            p = tk[idx, :K]
            assert (tk[idx, K:] == 0xFFFF).all()
            p = p[p != 0xFFFF]
            ok = inside[idx]
            nd = len(set(win[idx][ok].tolist()))
            assert len(p) == min(K, nd), (idx, len(p), nd)
            assert ok[p].all()
            wsel = win[idx][p]
            assert len(set(wsel.tolist())) == len(p)
            first = {}
            for q in np.nonzero(ok)[0]:
                first.setdefault(int(win[idx][q]), int(q))
            assert all(first[int(x)] == int(q) for x, q in zip(wsel, p))
            # approximate top-K: every left-out word scores at most tol above the lowest kept
            kept = set(wsel.tolist())
            lo = min(S[idx, p])
            for x, q in first.items():
                if x not in kept:
                    assert S[idx, q] <= lo + tol, (idx, x, S[idx, q], lo)
    enc.close()
    m.close()


def test_model_gradients_within_bf16_bounds(torch_cuda):
    """Every element of every layer's weight and bias gradient within the
    BF16 rounding bound of the CPU reference's."""
    torch = torch_cuda
    from mptc_gb300.model import ProposalModel, param_slices
    b = make_batch(torch)
    m = ProposalModel(seed=3)
    loss_gpu, g_gpu = m.grads(b["rgb_d"], b["w"], b["stb_d"], b["blocks_d"], b["cands_d"])
    B, C = b["cands"].shape
    p, Ws = layers(torch, m.params())
    hf, tf = mlp(torch, Ws, torch.tensor(block_features(b["frame"], b["stb"], b["blocks"], b["bw"])), [0, 1, 2])
    hg, tg = mlp(torch, Ws, torch.tensor(cand_features(b["cands"])), [3, 4])
    scores = (hf[:, None, :] * hg.view(B, C, 64)).sum(-1)
    loss = torch.nn.functional.cross_entropy(scores, torch.zeros(B, dtype=torch.long))
    loss.backward()
    assert abs(loss_gpu - float(loss.detach())) <= 2.0 ** -6 * abs(float(loss.detach())) + 1e-4
    sl, _ = param_slices()
    with torch.no_grad():
        for chain, ids in ((tf, [0, 1, 2]), (tg, [3, 4])):
            M = chain[-1][1].grad.abs()
            for pos in range(len(ids) - 1, -1, -1):
                li = ids[pos]
                inp, z = chain[pos]
                (a, e, shp), (c, d, _) = sl[li]
                w_bound = GRAD_TOL * (inp.abs().t() @ M) + 1e-7
                b_bound = GRAD_TOL * M.sum(0) + 1e-7
                gw = torch.tensor(g_gpu[a:e]).view(*shp)
                gb = torch.tensor(g_gpu[c:d])
                ew = (gw - p.grad[a:e].view(*shp)).abs()
                eb = (gb - p.grad[c:d]).abs()
                assert bool((ew <= w_bound).all()), (li, "weight", float((ew / w_bound).max()))
                assert bool((eb <= b_bound).all()), (li, "bias", float((eb / b_bound).max()))
                if pos > 0:  # magnitude of the gradient below: through |W| and the ReLU mask
                    M = (M @ bf(torch, Ws[li][0]).abs().t()) * (chain[pos - 1][1] > 0).float()
    m.close()


def test_candidate_errors_match_oracle(torch_cuda):
    """mptc_candidate_errors (the labels of the training examples) equals the
    oracle's refit error minus the block's stb error, INT_MAX where the refit
    swaps the endpoints, on random block / index-word pairs."""
    torch = torch_cuda
    import oracle
    from mptc_gb300.training import candidate_errors
    b = make_batch(torch, w=128, h=96, B=64, C=40, seed=8)
    err = candidate_errors(torch, b["rgb_d"], b["w"], 96, b["stb_d"], b["blocks_d"], b["cands_d"])
    for r, idx in enumerate(b["blocks"]):
        by, bx = divmod(int(idx), b["bw"])
        px = b["frame"][4 * by:4 * by + 4, 4 * bx:4 * bx + 4].reshape(48)
        orig = oracle.block_error(px, int(b["stb"][idx]))
        own = int(b["stb"][idx]) >> 32
        for c, word in enumerate(b["cands"][r]):
            if int(word) == own:
                assert err[r, c] == 0
                continue
            e, _, _, valid = oracle.refit(px, int(word))
            assert err[r, c] == (e - orig if valid else 0x7FFFFFFF), (r, c)


def test_training_reduces_loss_and_checkpoint_roundtrip(torch_cuda):
    torch = torch_cuda
    from mptc_gb300.model import ProposalModel
    b = make_batch(torch, B=256, C=16, seed=9)
    m = ProposalModel(seed=1)
    first = m.train_step(b["rgb_d"], b["w"], b["stb_d"], b["blocks_d"], b["cands_d"], lr=3e-3)
    for _ in range(60):
        last = m.train_step(b["rgb_d"], b["w"], b["stb_d"], b["blocks_d"], b["cands_d"], lr=3e-3)
    assert last < 0.5 * first, (first, last)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "m.bin")
        m.save(path)
        m2 = ProposalModel(seed=99)
        m2.load(path)
        np.testing.assert_array_equal(m.params(), m2.params())
        a = m.train_step(b["rgb_d"], b["w"], b["stb_d"], b["blocks_d"], b["cands_d"], lr=3e-3)
        c = m2.train_step(b["rgb_d"], b["w"], b["stb_d"], b["blocks_d"], b["cands_d"], lr=3e-3)
        # same parameters, moments and step count: the same update (the reported
        # loss is an atomic float sum, equal up to summation order)
        np.testing.assert_array_equal(m.params(), m2.params())
        assert abs(a - c) <= 1e-5 * abs(a)
        m2.close()
    m.close()


def quick_model(torch, frames, sa, steps, seed=2):
    from mptc_gb300.training import train_proposal
    dev = torch.device("cuda")
    model, losses, _ = train_proposal(torch, torch.from_numpy(frames).to(dev), sa, 5, 16, steps=steps, batch=1024,
                                      cands=16, lr=2e-3, seed=seed, per_frame=1024)
    return model, losses


def held_out_stats(torch, frames, sa, model, K):
    """Fallback rate and top-K recall of the plain search's accepted word on
    the inter frames of a stream."""
    from mptc_gb300._lib import check, lib
    from mptc_gb300.encoder import Encoder
    from mptc_gb300.training import accepted_inter, window_words
    n_, h, w, _ = frames.shape
    bw, bh = w // 4, h // 4
    n = bw * bh
    plain = Encoder(w, h, sa, 5, 16)
    learned = Encoder(w, h, sa, 5, 16)
    learned.set_model(model, K)
    dev = torch.device("cuda")
    fallback = inter = hit = total = 0
    prev = None
    for t, f in enumerate(frames):
        o = plain.encode_frame_host(f, is_intra=(t == 0), want_stb=True)
        learned.encode_frame_host(f, is_intra=(t == 0))
        if t > 0:
            st = learned.stats()
            fallback += st.n_fallback
            inter += n
            topk = torch.empty((n, 16), dtype=torch.int16, device=dev)
            check(lib().mptc_learned_proposals(
                learned.handle, torch.from_numpy(f.copy()).to(dev).data_ptr(),
                torch.from_numpy(o.stb.view(np.int64).copy()).to(dev).data_ptr(),
                torch.from_numpy(prev.view(np.int64).copy()).to(dev).data_ptr(), topk.data_ptr(),
                ctypes.c_void_p(0)), learned.handle)
            tk = topk.cpu().numpy().view(np.uint16).astype(np.int64)[:, :K]
            blocks, pos = accepted_inter(o.motion, bw, sa)
            win = window_words(prev, bw, bh, sa)[blocks]
            acc = win[np.arange(blocks.size), pos]
            prop = np.take_along_axis(win, np.where(tk[blocks] == 0xFFFF, 0, tk[blocks]), 1)
            prop[tk[blocks] == 0xFFFF] = -2
            hit += int((prop == acc[:, None]).any(1).sum())
            total += blocks.size
        prev = o.final.copy()
    plain.close()
    learned.close()
    return fallback / inter, hit / max(1, total)


def test_training_cli_trains_and_saves(torch_cuda, tmp_path, capsys):
    """python -m mptc_gb300.training: labels seeded 1080p frames with the
    exhaustive search, trains, prints one JSON line and writes weights that
    load back into a fresh model."""
    import json

    from mptc_gb300 import training
    from mptc_gb300.model import ProposalModel
    out = tmp_path / "proposal.bin"
    training.main(["--frames", "3", "--steps", "5", "--out", str(out)])
    info = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert info["steps"] == 5 and info["examples"] > 0 and np.isfinite(info["last_loss"]), info
    m = ProposalModel(seed=9)
    m.load(str(out))
    p = m.params()
    m.close()
    assert p.size > 0 and np.isfinite(p).all()


def test_trained_network_gains_over_untrained(torch_cuda):
    """On held-out frames (a separate seed), the trained network needs the
    exhaustive fallback for fewer blocks and proposes the exhaustive search's
    accepted word more often than the same network untrained."""
    torch = torch_cuda
    from mptc_gb300.model import ProposalModel
    sa, K = 8, 8
    train = StreamSpec(256, 256, 9, seed=600, n_squares=2, square_size=48).generate()
    held = StreamSpec(256, 256, 4, seed=601, n_squares=2, square_size=48).generate()
    model, losses = quick_model(torch, train, sa, steps=300)
    assert np.mean(losses[-20:]) < np.mean(losses[:20])
    untrained = ProposalModel(seed=2)
    fb_t, rec_t = held_out_stats(torch, held, sa, model, K)
    fb_u, rec_u = held_out_stats(torch, held, sa, untrained, K)
    assert fb_t < fb_u and rec_t > rec_u, (fb_t, fb_u, rec_t, rec_u)
    assert fb_t < 0.5 * fb_u, (fb_t, fb_u)
    model.close()
    untrained.close()


def test_learned_stream_is_valid(torch_cuda):
    """Accepted blocks meet the acceptance rule exactly (checked with the
    oracle's refit), unique blocks keep their stb block, motion codes point at
    the candidate whose index word was used, intra frames equal the plain path."""
    torch = torch_cuda
    import oracle
    from mptc_gb300.encoder import Encoder
    w, h, sa, thr = 192, 128, 6, 5
    frames = StreamSpec(w, h, 6, seed=31).generate()
    bw, bh = w // 4, h // 4
    plain = Encoder(w, h, sa, thr, 16)
    outs = [plain.encode_frame_host(f, want_stb=True) for f in frames]
    outs = [(o.stb.copy(), o.final.copy(), o.motion.copy(), o.unique.copy()) for o in outs]
    plain.close()
    m, _ = quick_model(torch, frames, sa, steps=60)
    for K in (4, 8, 16):
        enc = Encoder(w, h, sa, thr, 16)
        enc.set_model(m, K)
        prev = None
        for t, f in enumerate(frames):
            o = enc.encode_frame_host(f, want_stb=True)
            st = enc.stats()
            stb, fin, mot = o.stb, o.final, o.motion.reshape(-1, 2).astype(np.int64)
            if t == 0:
                np.testing.assert_array_equal(fin, outs[0][1])  # intra frame: exact path
            uniq = (mot[:, 0] == 255) & (mot[:, 1] == 255)
            np.testing.assert_array_equal(fin[uniq], stb[uniq])
            np.testing.assert_array_equal(o.unique, (stb[uniq] >> np.uint64(32)).astype(np.uint32))
            idx = np.arange(bw * bh)
            bx, by = idx % bw, idx // bw
            interp = (fin >> np.uint64(32)).astype(np.uint32)
            inter = ~uniq & (mot[:, 0] >= 128)
            if prev is not None:
                src = (by[inter] + mot[inter, 1] - 128 - sa) * bw + bx[inter] + mot[inter, 0] - 128 - sa
                np.testing.assert_array_equal(interp[inter], (prev[src] >> np.uint64(32)).astype(np.uint32))
            for k in np.nonzero(~uniq)[0]:
                y0, x0 = 4 * (k // bw), 4 * (k % bw)
                px = f[y0:y0 + 4, x0:x0 + 4].reshape(48)
                orig = oracle.block_error(px, int(stb[k]))
                if fin[k] == stb[k]:
                    continue  # identity candidate: err_diff 0
                err, _, _, valid = oracle.refit(px, int(interp[k]))
                assert valid and err - orig <= thr, (K, t, k, err, orig)
            assert st.n_inter + st.n_intra + st.n_unique == bw * bh
            prev = fin
        enc.close()
    m.close()


def test_learned_stream_decodes_bit_exactly(torch_cuda):
    """The learned path's output is an MPTC stream like any other: written by
    the host writer (pinned to the reference encoder's bytes) and rebuilt by
    the decoder (pinned to the reference decoder), it gives back the learned
    path's final blocks frame for frame."""
    torch = torch_cuda
    from mptc_gb300.decoder import decode_stream
    from mptc_gb300.encoder import Encoder
    from mptc_gb300.stream import write_stream
    w, h, sa, thr, ui = 256, 256, 8, 5, 4
    frames = StreamSpec(w, h, 8, seed=41).generate()
    m, _ = quick_model(torch, frames, sa, steps=40, seed=3)
    enc = Encoder(w, h, sa, thr, 16)
    enc.set_model(m, 8)
    learned = []
    for f in frames:
        o = enc.encode_frame_host(f)
        learned.append((o.final.copy(), o.motion.copy(), o.unique.copy()))
    enc.close()
    m.close()
    data = write_stream(learned, w, h, sa, ui)
    dec = decode_stream(data)
    assert len(dec) == len(frames)
    for k, d in enumerate(dec):
        np.testing.assert_array_equal(d, learned[k][0], err_msg=f"frame {k}")
