"""mptc_encode_frame_noalloc against mptc_encode_frame, through the C ABI.

The no-allocation entry point serves callers that may not allocate device
memory (hosts that reserve the whole device budget up front and forbid plugin
allocations; frame loops that cannot absorb the allocator's device-wide
synchronisation). It keeps its scratch in a fixed device array inside the
library, so the test also checks that a second call, which finds the first
call's leftovers in that array, still matches: an intra frame, then an inter
frame that searches the first call's output. Results must be bit-identical.
Collected last so that a failure here leaves every other test already run.
"""
import ctypes

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


def _noalloc(lib, cfg, w, h, rgb, prev, stb, fin, mot, uni, nu, stream):
    return lib.mptc_encode_frame_noalloc(
        ctypes.byref(cfg), w, h, rgb.data_ptr(), prev.data_ptr() if prev is not None else None,
        stb.data_ptr(), fin.data_ptr(), mot.data_ptr(), uni.data_ptr(), nu.data_ptr(),
        ctypes.c_void_p(stream.cuda_stream))


def _noisy_pair(w, h):
    """Two frames of noise with a drifting gradient band: nearly every block
    stays open after the inter search (more open blocks than the no-alloc
    scratch keeps sweep statistics for)."""
    rng = np.random.default_rng(77)
    frames = rng.integers(0, 256, size=(2, h, w, 3), dtype=np.uint8)
    yy, xx = np.mgrid[0:h, 0:w // 4]
    for k in range(2):
        g = (xx * 2 + yy + 3 * k) % 256
        frames[k, :, : w // 4, 0] = g
        frames[k, :, : w // 4, 1] = 255 - g
        frames[k, :, : w // 4, 2] = g // 2
    return frames


@pytest.mark.parametrize("w,h,sa,thr,content", [(256, 192, 8, 5, "stream"), (1920, 1080, 8, 5, "stream"),
                                                (512, 512, 8, 5, "noise")])
def test_noalloc_matches_encode_frame_two_calls(torch_cuda, w, h, sa, thr, content):
    torch = torch_cuda
    from mptc_gb300._lib import MPTC_OK, Config, lib
    from mptc_gb300.encoder import Encoder

    frames = StreamSpec(w, h, 2, seed=321).generate() if content == "stream" else _noisy_pair(w, h)
    dev = torch.device("cuda")
    n = (w // 4) * (h // 4)
    stream = torch.cuda.current_stream()

    def bufs():
        return dict(stb=torch.empty(n, dtype=torch.int64, device=dev),
                    fin=torch.empty(n, dtype=torch.int64, device=dev),
                    mot=torch.empty(2 * n, dtype=torch.uint8, device=dev),
                    uni=torch.empty(n, dtype=torch.int32, device=dev),
                    nu=torch.zeros(1, dtype=torch.int32, device=dev))

    # existing entry point: mptc_encode_frame on a context
    enc = Encoder(w, h, sa, thr, 16)
    ref = [bufs(), bufs()]
    rgb = [torch.from_numpy(f.copy()).to(dev) for f in frames]
    for k in range(2):
        prev = ref[k - 1]["fin"] if k else None
        b = ref[k]
        enc.encode_frame_device(rgb[k], prev, b["stb"], b["fin"], b["mot"], b["uni"], b["nu"], stream)
    torch.cuda.synchronize()
    enc.close()

    # no-allocation entry point, two calls in a row (intra, then inter)
    cfg = Config(sa, thr, 16, 0)
    got = [bufs(), bufs()]
    for k in range(2):
        prev = got[k - 1]["fin"] if k else None
        b = got[k]
        rc = _noalloc(lib(), cfg, w, h, rgb[k], prev, b["stb"], b["fin"], b["mot"], b["uni"], b["nu"], stream)
        assert rc == MPTC_OK
    torch.cuda.synchronize()

    for k in range(2):
        r, g = ref[k], got[k]
        cnt = int(r["nu"].item())
        assert int(g["nu"].item()) == cnt
        for key in ("stb", "fin", "mot"):
            np.testing.assert_array_equal(g[key].cpu().numpy(), r[key].cpu().numpy(),
                                          err_msg=f"call {k}: {key}")
        np.testing.assert_array_equal(g["uni"][:cnt].cpu().numpy(), r["uni"][:cnt].cpu().numpy())
    if content == "noise":  # both against the oracle on the inter frame
        import oracle
        ref_o = oracle.encode_stream(frames, sa, thr, 16, threads=8)
        np.testing.assert_array_equal(got[1]["fin"].cpu().numpy().view(np.uint64), ref_o[1].final)
        np.testing.assert_array_equal(got[1]["mot"].cpu().numpy(), ref_o[1].motion)


def test_noalloc_rejects_oversize_frame(torch_cuda):
    torch = torch_cuda
    from mptc_gb300._lib import MPTC_EINVAL, NOALLOC_MAX_BLOCKS, Config, lib
    w, h = 2048, 1032  # 512 x 258 = 132096 blocks > 131072
    assert (w // 4) * (h // 4) > NOALLOC_MAX_BLOCKS
    dev = torch.device("cuda")
    t = torch.empty(16, dtype=torch.int64, device=dev)
    cfg = Config(8, 5, 16, 0)
    rc = lib().mptc_encode_frame_noalloc(ctypes.byref(cfg), w, h, t.data_ptr(), None, None,
                                         t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(),
                                         ctypes.c_void_p(0))
    assert rc == MPTC_EINVAL
