"""Batched multi-stream encoding: every stream of a batch (mixed resolutions,
staggered intra frames) matches the same stream encoded alone, bit for bit,
and the autotuner keeps results unchanged."""
import numpy as np
import pytest

from mptc_gb300.synth import StreamSpec

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def single(frames, sa, thr, ii, flags):
    from mptc_gb300.encoder import Encoder
    h, w = frames.shape[1:3]
    enc = Encoder(w, h, sa, thr, ii)
    out = []
    for f, intra in zip(frames, flags):
        o = enc.encode_frame_host(f, is_intra=intra)
        out.append((o.final.copy(), o.motion.copy(), o.unique.copy()))
    enc.close()
    return out


def test_batch_matches_single_streams(torch_cuda):
    from mptc_gb300.batch import BatchEncoder
    sizes = [(256, 128), (128, 96), (320, 240), (64, 64)]
    nf = 5
    streams = [StreamSpec(w, h, nf, seed=50 + k, square_size=32).generate() for k, (w, h) in enumerate(sizes)]
    # stream k restarts with an intra frame at step k (staggered patterns)
    flags = [[f == 0 or f == k for f in range(nf)] for k in range(len(sizes))]
    ref = [single(streams[k], 6, 5, 16, flags[k]) for k in range(len(sizes))]
    b = BatchEncoder(sizes, 6, 5, 16)
    for f in range(nf):
        for k in range(len(sizes)):
            b.upload(k, streams[k][f])
        b.encode([flags[k][f] for k in range(len(sizes))])
        for k in range(len(sizes)):
            fin, mot, uni = b.fetch(k)
            np.testing.assert_array_equal(fin, ref[k][f][0], err_msg=f"stream {k} frame {f}")
            np.testing.assert_array_equal(mot, ref[k][f][1])
            np.testing.assert_array_equal(uni, ref[k][f][2])
    b.close()


def test_batch_autotune_keeps_results(torch_cuda):
    from mptc_gb300.batch import BatchEncoder
    sizes = [(192, 128), (192, 128)]
    streams = [StreamSpec(w, h, 3, seed=70 + k).generate() for k, (w, h) in enumerate(sizes)]
    flags = [True, False, False]
    ref = [single(streams[k], 8, 5, 16, flags) for k in range(2)]
    b = BatchEncoder(sizes, 8, 5, 16)
    for f in range(3):
        for k in range(2):
            b.upload(k, streams[k][f])
        if f == 1:
            t = b.autotune([False, False])
            assert t["inter_warps_per_cta"] in (2, 4) and t["intra_ctas_per_stream"] >= 0
        b.encode([flags[f]] * 2)
        for k in range(2):
            fin, mot, uni = b.fetch(k)
            np.testing.assert_array_equal(fin, ref[k][f][0])
            np.testing.assert_array_equal(mot, ref[k][f][1])
            np.testing.assert_array_equal(uni, ref[k][f][2])
    b.close()


def single_learned(frames, sa, thr, flags, model, K):
    from mptc_gb300.encoder import Encoder
    h, w = frames.shape[1:3]
    enc = Encoder(w, h, sa, thr, 16)
    enc.set_model(model, K)
    out = []
    for f, intra in zip(frames, flags):
        o = enc.encode_frame_host(f, is_intra=intra)
        out.append((o.final.copy(), o.motion.copy(), o.unique.copy()))
    enc.close()
    return out


@pytest.mark.parametrize("K", [8, 16])
def test_learned_batch_matches_single_streams(torch_cuda, K):
    """With a model attached, the batch runs each phase of the learned search
    as one launch over every stream (mixed resolutions, staggered intra
    frames); every stream's outputs equal the same stream encoded alone with
    the same model, before and after the autotuner changes the scoring's
    stage shape."""
    from mptc_gb300.batch import BatchEncoder
    from mptc_gb300.model import ProposalModel
    sizes = [(256, 128), (128, 96), (320, 240), (64, 64), (136, 72)]
    nf = 5
    streams = [StreamSpec(w, h, nf, seed=80 + k, square_size=32).generate() for k, (w, h) in enumerate(sizes)]
    flags = [[f == 0 or f == k for f in range(nf)] for k in range(len(sizes))]
    model = ProposalModel(seed=7)
    ref = [single_learned(streams[k], 8, 5, flags[k], model, K) for k in range(len(sizes))]
    b = BatchEncoder(sizes, 8, 5, 16)
    b.set_model(model, K)
    for f in range(nf):
        for k in range(len(sizes)):
            b.upload(k, streams[k][f])
        if f == 3:
            t = b.autotune([flags[k][f] for k in range(len(sizes))])
            assert t["score_rows_per_stage"] in (4, 8)
        b.encode([flags[k][f] for k in range(len(sizes))])
        for k in range(len(sizes)):
            fin, mot, uni = b.fetch(k)
            np.testing.assert_array_equal(fin, ref[k][f][0], err_msg=f"stream {k} frame {f}")
            np.testing.assert_array_equal(mot, ref[k][f][1])
            np.testing.assert_array_equal(uni, ref[k][f][2])
    b.close()
    model.close()


def test_batch_rejects_inter_first_frame(torch_cuda):
    from mptc_gb300._lib import MptcError
    from mptc_gb300.batch import BatchEncoder
    b = BatchEncoder([(64, 64)], 4, 5, 16)
    with pytest.raises(MptcError):
        b.encode([False])
    b.close()


@pytest.mark.parametrize("learned", [False, True])
def test_batch_run_matches_single_streams(torch_cuda, learned):
    """mptc_batch_encode_run (a run of frames of every stream: intra frames
    first on per-stream lanes, inter frames step by step) gives every stream's
    outputs of the same stream encoded alone, with and without a model, over
    two runs in a row (the streams continue across runs)."""
    torch = torch_cuda
    from mptc_gb300.batch import BatchEncoder
    from mptc_gb300.model import ProposalModel
    sizes = [(256, 128), (128, 96), (64, 64)]
    nf, runs = 6, 2
    streams = [StreamSpec(w, h, nf * runs, seed=90 + k, square_size=32).generate() for k, (w, h) in enumerate(sizes)]
    flags = [[f == 0 or f % 4 == k for f in range(nf * runs)] for k in range(len(sizes))]
    model = ProposalModel(seed=9) if learned else None
    ref = [single_learned(streams[k], 8, 5, flags[k], model, 8) if learned else single(streams[k], 8, 5, 16, flags[k])
           for k in range(len(sizes))]
    b = BatchEncoder(sizes, 8, 5, 16)
    if learned:
        b.set_model(model, 8)
    dev = torch.device("cuda")
    for r in range(runs):
        lo, hi = r * nf, (r + 1) * nf
        frames = [torch.from_numpy(streams[k][lo:hi].copy()).to(dev) for k in range(len(sizes))]
        fins = [torch.empty((nf, b.nblk(k)), dtype=torch.int64, device=dev) for k in range(len(sizes))]
        mots = [torch.empty((nf, 2 * b.nblk(k)), dtype=torch.uint8, device=dev) for k in range(len(sizes))]
        unis = [torch.empty((nf, b.nblk(k)), dtype=torch.int32, device=dev) for k in range(len(sizes))]
        nus = [torch.empty(nf, dtype=torch.int32, device=dev) for k in range(len(sizes))]
        b.encode_run(frames, fins, mots, unis, nus, [flags[k][lo:hi] for k in range(len(sizes))])
        torch.cuda.synchronize()
        for k in range(len(sizes)):
            for f in range(nf):
                np.testing.assert_array_equal(fins[k][f].cpu().numpy().view(np.uint64), ref[k][lo + f][0],
                                              err_msg=f"run {r} stream {k} frame {f}")
                np.testing.assert_array_equal(mots[k][f].cpu().numpy(), ref[k][lo + f][1])
                n = int(nus[k][f].item())
                np.testing.assert_array_equal(unis[k][f, :n].cpu().numpy().view(np.uint32), ref[k][lo + f][2])
    b.close()
    if model is not None:
        model.close()
