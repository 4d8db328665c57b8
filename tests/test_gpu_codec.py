"""GPU endpoint transform and GPU decoder against the reference.

* Coefficients computed on the GPU, coded by the host writer, give the
  reference encoder's stream bytes (golden.json "streams").
* The GPU decoder rebuilds the blocks the reference decoder's GetFrame
  rebuilds (golden "decoded", where GetFrame is defined) and, for every frame
  of the stream, the encoder's final blocks.
* At a full 2048x1280 size (1080p padded to 256-pixel multiples): encode on
  the GPU -> stream -> GPU decode returns the encoder's final blocks.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from mptc_gb300.synth import StreamSpec

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
STREAMS = json.load(open(os.path.join(GOLDEN, "golden.json")))["streams"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _oracle(case):
    spec = StreamSpec(**case["spec"])
    frames = spec.generate(case["first"], case["count"])
    res = oracle.encode_stream(frames, case["search_area"], case["threshold"], case["intra_interval"],
                               threads=os.cpu_count() or 1, want_psnr=False)
    return spec, res


@pytest.mark.parametrize("case", STREAMS, ids=[c["name"] for c in STREAMS])
def test_gpu_coefficients_give_reference_stream(torch_cuda, case):
    from mptc_gb300.decoder import endpoint_coefficients
    from mptc_gb300.stream import StreamWriter
    torch = torch_cuda
    spec, res = _oracle(case)
    n = (spec.width // 4) * (spec.height // 4)
    blocks = torch.empty(n, dtype=torch.int64, device="cuda")
    coeff = torch.empty(6 * n, dtype=torch.uint8, device="cuda")
    sw = StreamWriter(spec.width, spec.height, case["search_area"], case["unique_interval"], case["count"])
    for r in res:
        blocks.copy_(torch.from_numpy(r.final.view(np.int64)))
        endpoint_coefficients(spec.width, spec.height, blocks, coeff)
        sw.add_frame_coefficients(coeff.cpu().numpy(), r.motion, r.unique)
    data = sw.finish()
    sw.close()
    assert len(data) == case["size"]
    assert hashlib.sha256(data).hexdigest() == case["sha"]


@pytest.mark.parametrize("case", STREAMS, ids=[c["name"] for c in STREAMS])
def test_gpu_decoder_matches_reference_decoder(torch_cuda, case):
    from mptc_gb300.decoder import decode_stream
    from mptc_gb300.stream import write_stream
    spec, res = _oracle(case)
    data = write_stream(res, spec.width, spec.height, case["search_area"], case["unique_interval"])
    assert hashlib.sha256(data).hexdigest() == case["sha"]
    dec = decode_stream(data)
    ui = case["unique_interval"]
    assert len(dec) == (case["count"] // ui) * ui
    for k, g in enumerate(case["decoded"]):
        assert sha(dec[k]) == g, f"frame {k}: reference decoder"
    for k, d in enumerate(dec):
        np.testing.assert_array_equal(d, res[k].final, err_msg=f"frame {k}: encoder final blocks")


def test_gpu_decoder_flags_invalid_codes(torch_cuda):
    from mptc_gb300._lib import MptcError
    from mptc_gb300.decoder import Decoder
    w = h = 256
    n = (w // 4) * (h // 4)
    coeff = np.full(6 * n, 128, np.uint8)
    dec = Decoder(w, h, 4)
    # intra copy from a later block (block 0 referring forward)
    motion = np.full(2 * n, 255, np.uint8)
    motion[0], motion[1] = 7, 7
    dec.decode_frame(motion, coeff, np.zeros(n - 1, np.uint32))
    with pytest.raises(MptcError):
        dec.check()
    # inter copy without a previous frame is fine once a frame exists; unique count mismatch
    motion = np.full(2 * n, 255, np.uint8)
    dec.decode_frame(motion, coeff, np.zeros(5, np.uint32))
    with pytest.raises(MptcError):
        dec.check()
    # a valid all-unique frame clears
    dec.decode_frame(motion, coeff, np.arange(n, dtype=np.uint32))
    dec.check()
    dec.close()
    dec2 = Decoder(w, h, 4)
    motion = np.zeros(2 * n, np.uint8) | 0x80  # inter codes on the first frame
    dec2.decode_frame(motion, coeff, np.zeros(0, np.uint32))
    with pytest.raises(MptcError):
        dec2.check()
    dec2.close()


def test_gpu_encode_stream_decode_round_trip_2048x1280(torch_cuda):
    """Full-size property: GPU encoder -> GPU coefficients -> stream -> reader ->
    GPU decoder gives back the encoder's final blocks, frame for frame."""
    import torch
    from mptc_gb300.decoder import Decoder, endpoint_coefficients
    from mptc_gb300.encoder import Encoder
    from mptc_gb300.stream import StreamReader, StreamWriter
    w, h, nf, sa, ui = 2048, 1280, 4, 8, 2
    frames = StreamSpec(w, h, nf, seed=31, n_squares=4, square_size=128).generate()
    enc = Encoder(w, h, sa, 5, 16)
    n = (w // 4) * (h // 4)
    blocks = torch.empty(n, dtype=torch.int64, device="cuda")
    coeff = torch.empty(6 * n, dtype=torch.uint8, device="cuda")
    sw = StreamWriter(w, h, sa, ui, nf)
    finals = []
    for f in frames:
        o = enc.encode_frame_host(f)
        finals.append(o.final.copy())
        blocks.copy_(torch.from_numpy(o.final.view(np.int64)))
        endpoint_coefficients(w, h, blocks, coeff)
        sw.add_frame_coefficients(coeff.cpu().numpy(), o.motion, o.unique)
    data = sw.finish()
    sw.close()
    enc.close()
    rd = StreamReader(data)
    dec = Decoder(w, h, sa)
    k = 0
    for motion, c, unique in rd:
        out = dec.decode_frame(motion, c, unique)
        np.testing.assert_array_equal(out.cpu().numpy().view(np.uint64), finals[k], err_msg=f"frame {k}")
        k += 1
    dec.check()
    assert k == nf
    dec.close()
    rd.close()
