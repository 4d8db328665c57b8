"""GPU parity on the measured workloads at their full sizes, against records of
the unmodified reference encoder (tests/golden/configs.json, written by
``make_golden.py --configs``): every frame of the 120-frame 1080p stream
through the stream call the bench times, every frame of the 64-frame 720p
stream with its scene cut, one stream of each resolution of the mixed batch
through the batched encoder, the 2160p stream at the largest search area (63),
and the whole MPTC stream of the 720p workload (edge-padded to 1280x768) with
its blocks decoded back on the GPU as the reference decoder rebuilds them.
The decoded-block squared error the learned proposal's PSNR gate uses is
checked against the oracle on the same frames."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from mptc_gb300.synth import StreamSpec, pad_edge

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CONFIGS = json.load(open(os.path.join(GOLDEN, "configs.json")))
CASES = {c["name"]: c for c in CONFIGS["cases"]}
STREAMS = {c["name"]: c for c in CONFIGS["streams"]}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def frames_of(case):
    frames = StreamSpec(**case["spec"]).generate(case["first"], case["count"])
    assert [sha(f) for f in frames] == case["input_sha"], "synthetic inputs differ from the reference's"
    return frames


def check_frames(name, outs, with_stb=True):
    for k, (o, g) in enumerate(zip(outs, CASES[name]["frames"])):
        if with_stb:
            assert sha(o[0]) == g["stb"], f"{name} frame {k}: stb blocks"
        assert sha(o[1]) == g["final"], f"{name} frame {k}: final blocks"
        assert sha(o[2]) == g["motion"], f"{name} frame {k}: motion codes"
        assert sha(o[3]) == g["unique"], f"{name} frame {k}: unique palette"
    assert len(outs) == len(CASES[name]["frames"])


def test_gpu_1080p_120_frames_stream_call(torch_cuda):
    """The bench's workload: all 120 frames of the 1080p stream through
    mptc_encode_stream_device (intra frames on the second lane)."""
    from mptc_gb300.encoder import Encoder, intra_schedule
    torch = torch_cuda
    case = CASES["fhd1080_120f_sa8_thr5"]
    frames = frames_of(case)
    nf, h, w, _ = frames.shape
    enc = Encoder(w, h, case["search_area"], case["threshold"], case["intra_interval"])
    n = enc.nblk
    dev = torch.device("cuda")
    fin = torch.empty((nf, n), dtype=torch.int64, device=dev)
    mot = torch.empty((nf, 2 * n), dtype=torch.uint8, device=dev)
    uni = torch.empty((nf, n), dtype=torch.int32, device=dev)
    nu = torch.empty(nf, dtype=torch.int32, device=dev)
    enc.encode_stream_device(torch.from_numpy(frames).to(dev), fin, mot, uni, nu,
                             is_intra=intra_schedule(nf, case["intra_interval"]))
    torch.cuda.synchronize()
    enc.close()
    fin, mot, uni, nu = (t.cpu().numpy() for t in (fin, mot, uni, nu))
    outs = [(None, fin[k].view(np.uint64), mot[k], uni[k, :nu[k]].view(np.uint32)) for k in range(nf)]
    check_frames(case["name"], outs, with_stb=False)


def host_stream(frames, case):
    from mptc_gb300.encoder import Encoder
    h, w = frames.shape[1:3]
    enc = Encoder(w, h, case["search_area"], case["threshold"], case["intra_interval"])
    outs = []
    for f in frames:
        o = enc.encode_frame_host(f, want_stb=True)
        outs.append((o.stb.copy(), o.final.copy(), o.motion.copy(), o.unique.copy()))
    enc.close()
    return outs


def test_gpu_720p_64_frames_with_scene_cut(torch_cuda):
    case = CASES["hd720_64f_sa8_thr5"]
    check_frames(case["name"], host_stream(frames_of(case), case))


def test_gpu_2160p_largest_search_area(torch_cuda):
    """2160p at search area 63 (a 126 x 126-block inter window, 7,938-position
    intra window): the intra frame 0 and the inter frame 1."""
    case = CASES["uhd2160_sa63_thr5"]
    check_frames(case["name"], host_stream(frames_of(case), case))


def test_gpu_mixed_resolutions_batch(torch_cuda):
    """One stream of each mixed-batch resolution (854x480 generated at 856,
    720p, 1080p, 1440p) encoded together by the batched encoder."""
    from mptc_gb300.batch import BatchEncoder
    names = ["mixed_856x480_s1000", "mixed_1280x720_s1009", "mixed_1920x1080_s1018",
             "mixed_2560x1440_s1027"]
    streams = [frames_of(CASES[nm]) for nm in names]
    sizes = [(s.shape[2], s.shape[1]) for s in streams]
    c0 = CASES[names[0]]
    b = BatchEncoder(sizes, c0["search_area"], c0["threshold"], c0["intra_interval"])
    outs = [[] for _ in names]
    for f in range(c0["count"]):
        for k in range(len(names)):
            b.upload(k, streams[k][f])
        b.encode()  # the reference's schedule per stream
        for k in range(len(names)):
            fin, mot, uni = b.fetch(k)
            outs[k].append((None, fin.copy(), mot.copy(), uni.copy()))
    b.close()
    for k, nm in enumerate(names):
        check_frames(nm, outs[k], with_stb=False)


def test_gpu_720p_padded_stream_bytes_and_decode(torch_cuda):
    """The 64-frame 720p workload edge-padded to 1280x768: the GPU encoder's
    arrays through the host writer give the reference encoder's stream byte
    for byte, and the GPU decoder rebuilds the blocks the reference decoder's
    GetFrame rebuilds, frame by frame."""
    from mptc_gb300.decoder import decode_stream
    from mptc_gb300.encoder import Encoder
    from mptc_gb300.stream import write_stream
    case = STREAMS["hd720_pad1280x768_64f_sa8_thr5_ii16_ui8"]
    frames = pad_edge(StreamSpec(**case["spec"]).generate(0, case["count"]), case["pad"])
    assert (frames.shape[2], frames.shape[1]) == (case["width"], case["height"])
    assert [sha(f) for f in frames] == case["input_sha"]
    enc = Encoder(case["width"], case["height"], case["search_area"], case["threshold"], case["intra_interval"])
    out = enc.encode_stream_host(frames)
    enc.close()
    items = [(out.final[k].copy(), out.motion[k].copy(), out.unique[k, :out.n_unique[k]].copy())
             for k in range(case["count"])]
    data = write_stream(items, case["width"], case["height"], case["search_area"], case["unique_interval"])
    assert len(data) == case["size"]
    assert hashlib.sha256(data).hexdigest() == case["sha"]
    decoded = decode_stream(data)
    for k, d in enumerate(case["decoded"]):
        assert sha(decoded[k]) == d, f"decoded frame {k}"


def test_gpu_decoded_sse_matches_oracle(torch_cuda):
    """mptc_decoded_sse (decoded RGB565 palettes, the learned proposal's PSNR
    measure) against the oracle on the stb and final blocks of 1080p frames
    and of a noisy frame."""
    import ctypes

    from mptc_gb300._lib import check, lib
    from mptc_gb300.encoder import Encoder
    torch = torch_cuda
    case = CASES["fhd1080_120f_sa8_thr5"]
    frames = StreamSpec(**case["spec"]).generate(0, 3)
    rng = np.random.default_rng(5)
    noisy = rng.integers(0, 256, size=(1,) + frames.shape[1:], dtype=np.uint8)
    frames = np.concatenate([frames, noisy])
    h, w = frames.shape[1:3]
    enc = Encoder(w, h, 8, 5, 16)
    sse = torch.zeros(1, dtype=torch.int64, device="cuda")
    for k, f in enumerate(frames):
        o = enc.encode_frame_host(f, is_intra=(k == 0 or k == 3), want_stb=True)
        fd = torch.from_numpy(f).cuda()
        for blocks in (o.stb, o.final):
            bd = torch.from_numpy(blocks.view(np.int64).copy()).cuda()
            sse.zero_()
            check(lib().mptc_decoded_sse(fd.data_ptr(), w, h, bd.data_ptr(), sse.data_ptr(), ctypes.c_void_p(0)))
            torch.cuda.synchronize()
            assert int(sse.item()) == oracle.decoded_sse(f, blocks), f"frame {k}"
    enc.close()
