"""Learned candidate proposal: the GPU training kernels against a CPU
reference (torch fp32 with the BF16 operand rounding emulated), the forward
embeddings, training progress, checkpointing, and the validity of a stream
encoded with the proposal (every accepted block satisfies the reference's
acceptance rule; motion codes point at the chosen candidate)."""
import os
import tempfile

import numpy as np
import pytest

from mptc_gb300.synth import StreamSpec

pytestmark = pytest.mark.gpu

# Tolerances: operands are rounded to BF16 (8-bit mantissa) before every
# tensor-core product and activations/gradients are rounded between layers,
# so per-tensor agreement with the fp32 reference is checked as
# cosine similarity >= 0.99 and relative L2 error <= 0.08.
COS_MIN, REL_MAX = 0.99, 0.08


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def block_features(frame, stb, blocks, bw):
    X = np.zeros((len(blocks), 64), np.float32)
    for r, idx in enumerate(blocks):
        by, bx = divmod(int(idx), bw)
        px = frame[4 * by:4 * by + 4, 4 * bx:4 * bx + 4].reshape(16, 3).astype(np.float32) / 255.0
        X[r, :48] = px.reshape(48)
        for k, ep in enumerate([int(stb[idx]) & 0xFFFF, (int(stb[idx]) >> 16) & 0xFFFF]):
            X[r, 48 + 3 * k:51 + 3 * k] = [(ep >> 11) / 31.0, ((ep >> 5) & 63) / 63.0, (ep & 31) / 31.0]
    return X


def cand_features(words):
    w = np.asarray(words, np.uint64).reshape(-1)
    return ((w[:, None] >> np.arange(32, dtype=np.uint64)[None, :]) & np.uint64(1)).astype(np.float32)


def torch_model(torch, params, X, Xc, B, C):
    from mptc_gb300.model import param_slices
    sl, _ = param_slices()
    p = torch.tensor(params, dtype=torch.float32, requires_grad=True)
    bf = lambda t: t.to(torch.bfloat16).to(torch.float32)  # noqa: E731
    Ws = [(p[a:b].view(*shp), p[c:d]) for (a, b, shp), (c, d, _) in sl]
    h = torch.tensor(X)
    for li in range(3):
        h = bf(h) @ bf(Ws[li][0]) + Ws[li][1]
        if li < 2:
            h = torch.relu(h)
    g = torch.tensor(Xc)
    for li in range(3, 5):
        g = bf(g) @ bf(Ws[li][0]) + Ws[li][1]
        if li == 3:
            g = torch.relu(g)
    scores = (h[:, None, :] * g.view(B, C, 64)).sum(-1)
    loss = torch.nn.functional.cross_entropy(scores, torch.zeros(B, dtype=torch.long))
    return p, h, g, loss


def agree(a, b):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30))
    rel = float(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30))
    return cos, rel


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
    return dict(frame=frames[1], stb=o1.stb, blocks=blocks, cands=cands, bw=bw, w=w,
                rgb_d=torch.from_numpy(frames[1].copy()).to(dev),
                stb_d=torch.from_numpy(o1.stb.view(np.int64)).to(dev),
                blocks_d=torch.from_numpy(blocks).to(dev),
                cands_d=torch.from_numpy(cands.view(np.int32)).to(dev))


def test_model_gradients_match_cpu_reference(torch_cuda):
    torch = torch_cuda
    from mptc_gb300.model import ProposalModel, param_slices
    b = make_batch(torch)
    m = ProposalModel(seed=3)
    params = m.params()
    loss_gpu, g_gpu = m.grads(b["rgb_d"], b["w"], b["stb_d"], b["blocks_d"], b["cands_d"])
    B, C = b["cands"].shape
    X = block_features(b["frame"], b["stb"], b["blocks"], b["bw"])
    Xc = cand_features(b["cands"])
    p, _, _, loss = torch_model(torch, params, X, Xc, B, C)
    loss.backward()
    g_ref = p.grad.numpy()
    assert abs(loss_gpu - float(loss.detach())) <= 0.02 * abs(float(loss.detach())) + 1e-4
    sl, _ = param_slices()
    scale = np.linalg.norm(g_ref)
    for li, ((a, e, _), (c, d, _)) in enumerate(sl):
        for lo, hi in ((a, e), (c, d)):
            if np.linalg.norm(g_ref[lo:hi]) < 1e-6 * scale:
                # e.g. the last candidate bias: softmax is invariant to adding one
                # vector to every candidate embedding, so its true gradient is 0
                assert np.linalg.norm(g_gpu[lo:hi]) < 1e-3 * scale, (li, lo)
                continue
            cos, rel = agree(g_gpu[lo:hi], g_ref[lo:hi])
            assert cos >= COS_MIN and rel <= REL_MAX, (li, lo, cos, rel)
    m.close()


def test_model_embeddings_match_cpu_reference(torch_cuda):
    torch = torch_cuda
    from mptc_gb300.model import ProposalModel
    b = make_batch(torch, B=64, C=2)
    m = ProposalModel(seed=4)
    B = b["blocks"].size
    F = torch.empty((B, 64), dtype=torch.float32, device="cuda")
    G = torch.empty((B, 64), dtype=torch.float32, device="cuda")
    words = b["cands_d"][:, 0].contiguous()
    m.embed(b["rgb_d"], b["w"], b["stb_d"], b["blocks_d"], B, F, words, 1, B, G)
    torch.cuda.synchronize()
    X = block_features(b["frame"], b["stb"], b["blocks"], b["bw"])
    Xc = cand_features(b["cands"][:, 0])
    _, h, g, _ = torch_model(torch, m.params(), X, np.repeat(Xc, 1, axis=0), B, 1)
    for got, ref in ((F.cpu().numpy(), h.detach().numpy()), (G.cpu().numpy(), g.detach().numpy())):
        cos, rel = agree(got, ref)
        assert cos >= COS_MIN and rel <= REL_MAX, (cos, rel)
    m.close()


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


def test_learned_stream_is_valid(torch_cuda):
    """Accepted blocks meet the acceptance rule exactly (checked with the
    oracle's refit), unique blocks keep their stb block, motion codes point at
    the candidate whose index word was used, intra frames equal the plain path."""
    torch = torch_cuda
    import oracle
    from mptc_gb300.encoder import Encoder
    from mptc_gb300.model import ProposalModel, sample_examples
    w, h, sa, thr = 192, 128, 6, 5
    frames = StreamSpec(w, h, 6, seed=31).generate()
    bw, bh = w // 4, h // 4
    # quick training on the plain search's decisions of the same stream
    plain = Encoder(w, h, sa, thr, 16)
    outs = [plain.encode_frame_host(f, want_stb=True) for f in frames]
    outs = [(o.stb.copy(), o.final.copy(), o.motion.copy(), o.unique.copy()) for o in outs]
    plain.close()
    m = ProposalModel(seed=2)
    rng = np.random.default_rng(0)
    dev = torch.device("cuda")
    for step in range(40):
        t = 1 + step % (len(frames) - 1)
        ex = sample_examples(rng, bw, bh, sa, outs[t][2], outs[t - 1][1], 256, 16)
        if ex is None:
            continue
        m.train_step(torch.from_numpy(frames[t].copy()).to(dev), w,
                     torch.from_numpy(outs[t][0].view(np.int64)).to(dev),
                     torch.from_numpy(ex.blocks).to(dev), torch.from_numpy(ex.cands.view(np.int32)).to(dev))
    enc = Encoder(w, h, sa, thr, 16)
    enc.set_model(m, 8)
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
        # acceptance rule, exactly, on every accepted block
        for k in np.nonzero(~uniq)[0]:
            y0, x0 = 4 * (k // bw), 4 * (k % bw)
            px = f[y0:y0 + 4, x0:x0 + 4].reshape(48)
            orig = oracle.block_error(px, int(stb[k]))
            if fin[k] == stb[k]:
                continue  # identity candidate: err_diff 0
            err, _, _, valid = oracle.refit(px, int(interp[k]))
            assert valid and err - orig <= thr, (t, k, err, orig)
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
    from mptc_gb300.model import ProposalModel, sample_examples
    from mptc_gb300.stream import write_stream
    w, h, sa, thr, ui = 256, 256, 8, 5, 4
    frames = StreamSpec(w, h, 8, seed=41).generate()
    bw, bh = w // 4, h // 4
    plain = Encoder(w, h, sa, thr, 16)
    outs = [plain.encode_frame_host(f, want_stb=True) for f in frames]
    outs = [(o.stb.copy(), o.final.copy(), o.motion.copy()) for o in outs]
    plain.close()
    m = ProposalModel(seed=3)
    rng = np.random.default_rng(1)
    dev = torch.device("cuda")
    for step in range(30):
        t = 1 + step % (len(frames) - 1)
        ex = sample_examples(rng, bw, bh, sa, outs[t][2], outs[t - 1][1], 256, 16)
        if ex is None:
            continue
        m.train_step(torch.from_numpy(frames[t].copy()).to(dev), w,
                     torch.from_numpy(outs[t][0].view(np.int64)).to(dev),
                     torch.from_numpy(ex.blocks).to(dev), torch.from_numpy(ex.cands.view(np.int32)).to(dev))
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
