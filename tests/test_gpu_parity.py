"""GPU parity: the CUDA path (through the C ABI) against the oracle and against
the golden vectors recorded from the reference encoder. Integer/byte outputs
must be bit-identical."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from mptc_gb300.synth import StreamSpec

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def gpu_stream(frames, sa, thr, ii, want_stb=True):
    from mptc_gb300.encoder import Encoder
    n, h, w, _ = frames.shape
    enc = Encoder(w, h, sa, thr, ii)
    outs = []
    for f in frames:
        o = enc.encode_frame_host(f, want_stb=want_stb)
        outs.append((o.stb.copy() if o.stb is not None else None, o.final.copy(), o.motion.copy(),
                     o.unique.copy()))
    enc.close()
    return outs


CASES = json.load(open(os.path.join(GOLDEN, "golden.json")))["cases"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_gpu_matches_reference_golden(torch_cuda, case):
    spec = StreamSpec(**case["spec"])
    frames = spec.generate(case["first"], case["count"])
    assert [sha(f) for f in frames] == case["input_sha"]
    outs = gpu_stream(frames, case["search_area"], case["threshold"], case["intra_interval"])
    for k, ((stb, fin, mot, uni), g) in enumerate(zip(outs, case["frames"])):
        assert sha(stb) == g["stb"], f"frame {k}: stb blocks"
        assert sha(fin) == g["final"], f"frame {k}: final blocks"
        assert sha(mot) == g["motion"], f"frame {k}: motion codes"
        assert sha(uni) == g["unique"], f"frame {k}: unique palette"


STREAMS = json.load(open(os.path.join(GOLDEN, "golden.json")))["streams"]


@pytest.mark.parametrize("case", STREAMS, ids=[c["name"] for c in STREAMS])
def test_gpu_stream_bytes_match_reference(torch_cuda, case):
    """CUDA encoder arrays -> host stream writer -> the reference encoder's
    stream, byte for byte."""
    from mptc_gb300.stream import write_stream
    spec = StreamSpec(**case["spec"])
    frames = spec.generate(case["first"], case["count"])
    outs = gpu_stream(frames, case["search_area"], case["threshold"], case["intra_interval"],
                      want_stb=False)
    data = write_stream([o[1:] for o in outs], spec.width, spec.height, case["search_area"],
                        case["unique_interval"])
    assert len(data) == case["size"]
    assert hashlib.sha256(data).hexdigest() == case["sha"]


@pytest.mark.parametrize("key", ["adv_sa4_thr5_ii16", "adv_sa2_thr0_ii1"])
def test_gpu_matches_reference_adversarial(torch_cuda, key):
    z = np.load(os.path.join(GOLDEN, f"{key}.npz"))
    sa, thr, ii = (int(v) for v in z["params"])
    outs = gpu_stream(z["frames"], sa, thr, ii)
    np.testing.assert_array_equal(np.stack([o[0] for o in outs]), z["stb"])
    np.testing.assert_array_equal(np.stack([o[1] for o in outs]), z["final"])
    np.testing.assert_array_equal(np.stack([o[2] for o in outs]), z["motion"])
    np.testing.assert_array_equal(np.concatenate([o[3] for o in outs]), z["unique"])


@pytest.mark.parametrize("w,h,sa,thr,ii,seed", [
    (64, 64, 4, 5, 16, 1), (128, 64, 8, 0, 2, 2), (96, 96, 3, 10, 1, 3), (256, 128, 12, 5, 4, 4),
    (64, 32, 63, 5, 2, 5), (40, 200, 5, -3, 3, 6), (4, 4, 1, 5, 2, 7), (8, 12, 2, 100, 2, 8)])
def test_gpu_matches_oracle_params(torch_cuda, w, h, sa, thr, ii, seed):
    frames = StreamSpec(w, h, 4, seed=seed, square_size=max(4, min(w, h) // 4)).generate()
    outs = gpu_stream(frames, sa, thr, ii)
    ref = oracle.encode_stream(frames, sa, thr, ii)
    for k, (o, r) in enumerate(zip(outs, ref)):
        np.testing.assert_array_equal(o[0], r.stb, err_msg=f"frame {k} stb")
        np.testing.assert_array_equal(o[1], r.final, err_msg=f"frame {k} final")
        np.testing.assert_array_equal(o[2], r.motion, err_msg=f"frame {k} motion")
        np.testing.assert_array_equal(o[3], r.unique, err_msg=f"frame {k} unique")


@pytest.mark.parametrize("sa,thr", [(8, 5), (8, 400), (5, 60), (2, 5)])
def test_gpu_matches_oracle_noisy(torch_cuda, sa, thr):
    """Noise on the left half (every window word distinct: the inter search's
    run table overflows and the blocks are searched one by one) beside a
    slowly moving gradient on the right (runs share their windows)."""
    rng = np.random.default_rng(100 + sa + thr)
    n, h, w = 3, 64, 128
    frames = rng.integers(0, 256, size=(n, h, w, 3), dtype=np.uint8)
    yy, xx = np.mgrid[0:h, 0:w // 2]
    for k in range(n):
        g = (xx * 3 + yy * 2 + 5 * k) % 256
        frames[k, :, w // 2:, 0] = g
        frames[k, :, w // 2:, 1] = (g // 2 + 40) % 256
        frames[k, :, w // 2:, 2] = 255 - g
    outs = gpu_stream(frames, sa, thr, 16)
    ref = oracle.encode_stream(frames, sa, thr, 16)
    for k, (o, r) in enumerate(zip(outs, ref)):
        np.testing.assert_array_equal(o[1], r.final, err_msg=f"frame {k} final")
        np.testing.assert_array_equal(o[2], r.motion, err_msg=f"frame {k} motion")
        np.testing.assert_array_equal(o[3], r.unique, err_msg=f"frame {k} unique")


def test_gpu_intra_1080p_matches_oracle(torch_cuda):
    """A full 1080p intra frame: ~129k blocks chained through the causal window."""
    frames = StreamSpec(1920, 1080, 1, seed=77).generate()
    outs = gpu_stream(frames, 8, 5, 16)
    r = oracle.reencode(frames[0], oracle.dxt1_encode(frames[0]), None, 8, 5, want_psnr=False)
    np.testing.assert_array_equal(outs[0][1], r.final)
    np.testing.assert_array_equal(outs[0][2], r.motion)
    np.testing.assert_array_equal(outs[0][3], r.unique)


def test_gpu_device_api_matches_host_api(torch_cuda):
    torch = torch_cuda
    from mptc_gb300.encoder import Encoder
    frames = StreamSpec(256, 128, 3, seed=9).generate()
    host = gpu_stream(frames, 8, 5, 16)
    enc = Encoder(256, 128, 8, 5, 16)
    n = enc.nblk
    dev = torch.device("cuda")
    fin = [torch.empty(n, dtype=torch.int64, device=dev) for _ in range(2)]
    stb = torch.empty(n, dtype=torch.int64, device=dev)
    mot = torch.empty(2 * n, dtype=torch.uint8, device=dev)
    uni = torch.empty(n, dtype=torch.int32, device=dev)
    nu = torch.zeros(1, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream()
    for k, f in enumerate(frames):
        rgb = torch.from_numpy(f.copy()).to(dev)
        prev = None if k == 0 else fin[(k - 1) % 2]
        enc.encode_frame_device(rgb, prev, stb, fin[k % 2], mot, uni, nu, s)
        torch.cuda.synchronize()
        cnt = int(nu.item())
        np.testing.assert_array_equal(fin[k % 2].cpu().numpy().view(np.uint64), host[k][1])
        np.testing.assert_array_equal(mot.cpu().numpy(), host[k][2])
        np.testing.assert_array_equal(uni[:cnt].cpu().numpy().view(np.uint32), host[k][3])
        st = enc.stats(s)
        assert st.n_unique == cnt and st.n_inter + st.n_intra + st.n_unique == n
    enc.close()


@pytest.mark.parametrize("pinned", [True, False])
def test_gpu_stream_host_matches_frame_host(torch_cuda, pinned):
    """mptc_encode_stream_host (pipelined copies with pinned buffers, frame by
    frame with pageable ones) gives the per-frame host call's results, and the
    stream continues across calls."""
    torch = torch_cuda
    from mptc_gb300.encoder import Encoder, StreamOutput
    frames = StreamSpec(256, 128, 7, seed=21, n_squares=3, square_size=40, speed_min=2,
                        speed_max=5).generate()
    ref = gpu_stream(frames, 8, 5, 3)
    enc = Encoder(256, 128, 8, 5, 3)
    n = enc.nblk

    def buf(shape, dtype):
        t = torch.zeros(shape, dtype=dtype)
        return (t.pin_memory() if pinned else t).numpy()

    src = buf(frames.shape, torch.uint8)
    src[:] = frames
    out = StreamOutput(buf((7, n), torch.int64).view(np.uint64), buf((7, 2 * n), torch.uint8),
                       buf((7, n), torch.int32).view(np.uint32), buf((7,), torch.int32).view(np.uint32))
    for a, b in ((0, 4), (4, 7)):
        enc.encode_stream_host(src[a:b], out=StreamOutput(out.final[a:b], out.motion[a:b], out.unique[a:b],
                                                          out.n_unique[a:b]))
    for k in range(7):
        o = out.frame(k)
        np.testing.assert_array_equal(o.final, ref[k][1], err_msg=f"frame {k} final")
        np.testing.assert_array_equal(o.motion, ref[k][2], err_msg=f"frame {k} motion")
        np.testing.assert_array_equal(o.unique, ref[k][3], err_msg=f"frame {k} unique")
    enc.close()


def test_gpu_stream_host_ring_wraps(torch_cuda):
    """A pinned host run longer than the device frame ring (24 slots), with
    intra frames every 5th frame on the second lane: every frame matches the
    per-frame host call."""
    torch = torch_cuda
    from mptc_gb300.encoder import Encoder, StreamOutput
    nf = 31
    frames = StreamSpec(128, 64, nf, seed=29, n_squares=2, square_size=24, speed_min=1,
                        speed_max=4).generate()
    ref = gpu_stream(frames, 4, 5, 5)
    enc = Encoder(128, 64, 4, 5, 5)
    n = enc.nblk
    src = torch.from_numpy(frames).pin_memory().numpy()
    out = StreamOutput(torch.zeros((nf, n), dtype=torch.int64).pin_memory().numpy().view(np.uint64),
                       torch.zeros((nf, 2 * n), dtype=torch.uint8).pin_memory().numpy(),
                       torch.zeros((nf, n), dtype=torch.int32).pin_memory().numpy().view(np.uint32),
                       torch.zeros(nf, dtype=torch.int32).pin_memory().numpy().view(np.uint32))
    enc.encode_stream_host(src, out=out)
    for k in range(nf):
        o = out.frame(k)
        np.testing.assert_array_equal(o.final, ref[k][1], err_msg=f"frame {k} final")
        np.testing.assert_array_equal(o.motion, ref[k][2], err_msg=f"frame {k} motion")
        np.testing.assert_array_equal(o.unique, ref[k][3], err_msg=f"frame {k} unique")
    enc.close()


def test_gpu_stream_device_matches_frame_host(torch_cuda):
    """mptc_encode_stream_device (intra frames on the second lane, concurrent
    with the inter frames before them) gives the per-frame results, across
    calls that start with an intra or an inter frame, and the stream then
    continues through the per-frame host call."""
    torch = torch_cuda
    from mptc_gb300.encoder import Encoder
    frames = StreamSpec(256, 128, 9, seed=23, n_squares=3, square_size=40, speed_min=2,
                        speed_max=5).generate()
    ref = gpu_stream(frames, 8, 5, 3)  # intra frames 0, 3, 6
    enc = Encoder(256, 128, 8, 5, 3)
    n, dev = enc.nblk, torch.device("cuda")
    src = torch.from_numpy(frames).to(dev)
    fin = torch.zeros((8, n), dtype=torch.int64, device=dev)
    mot = torch.zeros((8, 2 * n), dtype=torch.uint8, device=dev)
    uni = torch.zeros((8, n), dtype=torch.int32, device=dev)
    nu = torch.zeros(8, dtype=torch.int32, device=dev)
    for a, b in ((0, 5), (5, 8)):  # the second call starts with an inter frame
        enc.encode_stream_device(src[a:b], fin[a:b], mot[a:b], uni[a:b], nu[a:b],
                                 stream=torch.cuda.current_stream())
    fin, mot, uni, nu = (t.cpu().numpy() for t in (fin, mot, uni, nu))
    for k in range(8):
        np.testing.assert_array_equal(fin[k].view(np.uint64), ref[k][1], err_msg=f"frame {k} final")
        np.testing.assert_array_equal(mot[k], ref[k][2], err_msg=f"frame {k} motion")
        np.testing.assert_array_equal(uni[k, : nu[k]].view(np.uint32), ref[k][3], err_msg=f"frame {k} unique")
    o = enc.encode_frame_host(frames[8])  # an inter frame on the run's last frame
    np.testing.assert_array_equal(o.final, ref[8][1])
    np.testing.assert_array_equal(o.motion, ref[8][2])
    enc.close()


def test_gpu_rejects_bad_arguments(torch_cuda):
    from mptc_gb300._lib import MptcError
    from mptc_gb300.encoder import Encoder
    with pytest.raises(MptcError):
        Encoder(30, 32)
    with pytest.raises(MptcError):
        Encoder(32, 32, search_area=64)
    enc = Encoder(32, 32)
    with pytest.raises(MptcError):  # an inter frame needs a previous frame
        enc.encode_frame_host(np.zeros((32, 32, 3), np.uint8), is_intra=False)
    with pytest.raises(MptcError):  # the same for a run that starts with one
        enc.encode_stream_host(np.zeros((2, 32, 32, 3), np.uint8), is_intra=[False, False])
    torch = torch_cuda
    z = torch.zeros((2, 32, 32, 3), dtype=torch.uint8, device="cuda")
    outs = (torch.zeros((2, 64), dtype=torch.int64, device="cuda"), torch.zeros((2, 128), dtype=torch.uint8, device="cuda"),
            torch.zeros((2, 64), dtype=torch.int32, device="cuda"), torch.zeros(2, dtype=torch.int32, device="cuda"))
    with pytest.raises(MptcError):
        enc.encode_stream_device(z, *outs, is_intra=[False, True])
    with pytest.raises(ValueError):  # one frame's final blocks for a run of two
        enc.encode_stream_device(z, outs[0][:1], *outs[1:], is_intra=[True, False])
    with pytest.raises(ValueError):  # 4-byte words where the final blocks are 8
        enc.encode_stream_device(z, outs[2], outs[1], outs[2], outs[3], is_intra=[True, False])
    enc.encode_stream_device(z[:0], *(o[:0] for o in outs), is_intra=[])  # an empty run does nothing
    enc.encode_stream_device(z, *outs, is_intra=[True, False])
    assert (outs[0].cpu().numpy() != 0).any()
    enc.close()


def test_gpu_deterministic_and_consistent_2160p(torch_cuda):
    """Full-size properties at 3840x2160 (the oracle is too slow here): two runs
    agree bit for bit, unique blocks keep their stb block and feed the palette
    in raster order, and every match points at a block whose final interp is
    the chosen one."""
    frames = StreamSpec(3840, 2160, 2, period_min=128, period_max=1024, n_squares=16,
                        square_size=256, speed_min=1, speed_max=4, seed=1000).generate()
    a = gpu_stream(frames, 8, 5, 16)
    b = gpu_stream(frames, 8, 5, 16)
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            np.testing.assert_array_equal(u, v)
    bw, bh = 960, 540
    sa = 8
    prev_final = None
    for stb, fin, mot, uni in a:
        m = mot.reshape(-1, 2).astype(np.int64)
        uniq = (m[:, 0] == 255) & (m[:, 1] == 255)
        np.testing.assert_array_equal(fin[uniq], stb[uniq])
        np.testing.assert_array_equal(uni, (stb[uniq] >> np.uint64(32)).astype(np.uint32))
        idx = np.arange(bw * bh)
        bx, by = idx % bw, idx // bw
        interp = (fin >> np.uint64(32)).astype(np.uint32)
        inter = ~uniq & (m[:, 0] >= 128)
        intra = ~uniq & (m[:, 0] < 128)
        if prev_final is not None:
            src = (by[inter] + (m[inter, 1] - 128) - sa) * bw + bx[inter] + (m[inter, 0] - 128) - sa
            np.testing.assert_array_equal(interp[inter], (prev_final[src] >> np.uint64(32)).astype(np.uint32))
        else:
            assert not inter.any()
        src = (by[intra] + m[intra, 1] - (2 * sa - 1)) * bw + bx[intra] + m[intra, 0] - sa
        assert (src < idx[intra]).all()  # causal
        np.testing.assert_array_equal(interp[intra], interp[src])
        prev_final = fin


@pytest.mark.parametrize("sweeps", [-1, 1, 2, 32])
def test_gpu_intra_pass_same_for_any_sweep_count(torch_cuda, sweeps):
    """The inter frames' intra pass gives the reference's result whether the
    fixed-point sweeps converge (many sweeps), stop early and hand over to the
    dataflow kernel (1-2 sweeps) or are skipped (dataflow only)."""
    from mptc_gb300.encoder import Encoder
    spec = StreamSpec(256, 192, 4, seed=90, n_squares=3, square_size=48, speed_min=3, speed_max=5)
    frames = spec.generate()
    ref = oracle.encode_stream(frames, 6, 2, 16)
    enc = Encoder(256, 192, 6, 2, 16, intra_sweeps=sweeps)
    for k, f in enumerate(frames):
        o = enc.encode_frame_host(f)
        np.testing.assert_array_equal(o.final, ref[k].final, err_msg=f"frame {k} final")
        np.testing.assert_array_equal(o.motion, ref[k].motion, err_msg=f"frame {k} motion")
        np.testing.assert_array_equal(o.unique, ref[k].unique, err_msg=f"frame {k} unique")
    enc.close()
