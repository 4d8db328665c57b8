"""Host stream writer (include/mptc_host.h) against whole MPTC streams written
by the reference encoder (golden.json "streams": SHA-256 of the bytes of
CompressMultiUnique, codec/codec.cpp:1307-1532, over the same frames).

The frame arrays fed to the writer come from the oracle here; the GPU test in
test_gpu_parity.py feeds the CUDA encoder's arrays to the same writer."""
import hashlib
import json
import os
import struct

import numpy as np
import pytest

import oracle
from mptc_gb300.stream import StreamWriter, write_stream
from mptc_gb300.synth import StreamSpec
from mptc_gb300._lib import MptcError

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
STREAMS = json.load(open(os.path.join(GOLDEN, "golden.json")))["streams"]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("case", STREAMS, ids=[c["name"] for c in STREAMS])
def test_oracle_arrays_give_reference_stream(case):
    spec = StreamSpec(**case["spec"])
    frames = spec.generate(case["first"], case["count"])
    assert [sha(f) for f in frames] == case["input_sha"]
    res = oracle.encode_stream(frames, case["search_area"], case["threshold"],
                               case["intra_interval"], threads=os.cpu_count() or 1, want_psnr=False)
    data = write_stream(res, spec.width, spec.height, case["search_area"], case["unique_interval"])
    assert data[:34].hex() == case["header"]
    assert len(data) == case["size"]
    assert hashlib.sha256(data).hexdigest() == case["sha"]


def test_header_fields_and_group_layout():
    """Header per codec/codec.cpp:1354-1367 and :1514-1520; one group record
    per unique_interval frames, trailing frames left out."""
    w, h, n = 256, 256, 5
    nb = (w // 4) * (h // 4)
    rng = np.random.default_rng(3)
    final = rng.integers(0, 2**63, nb, dtype=np.uint64)
    motion = np.full(2 * nb, 255, np.uint8)
    uniq = np.arange(7, dtype=np.uint32)
    sw = StreamWriter(w, h, 300 % 64, 2, n)  # search area fits a byte
    for _ in range(n):
        sw.add_frame(final, motion, uniq)
    mb, ep = sw.frame_sizes()
    data = sw.finish()
    sw.close()
    hh, ww, ui, sa, groups = struct.unpack_from("<IIBBI", data, 0)
    assert (hh, ww, ui, sa, groups) == (h, w, 2, 300 % 64, n // 2)
    max_unique, max_pal, max_mo, max_y, max_c = struct.unpack_from("<5I", data, 14)
    assert max_unique == 2 * 4 * uniq.size  # palette BYTES of a group
    assert max_mo == mb and max_y == max(ep[0], ep[2]) and max_c == max(ep[1], ep[3])
    # walk the groups: [u32 palette size][palette][u32 count][2 frame records]
    off = 34
    for _ in range(groups):
        (psz,) = struct.unpack_from("<I", data, off)
        assert psz <= max_pal
        off += 4 + psz
        (cnt,) = struct.unpack_from("<I", data, off)
        assert cnt == 2 * 4 * uniq.size
        off += 4
        for _ in range(2):
            nu, msz = struct.unpack_from("<II", data, off)
            assert nu == uniq.size and msz == mb
            off += 8 + msz
            for k in range(4):
                (esz,) = struct.unpack_from("<I", data, off)
                assert esz == ep[k]
                off += 4 + esz
    assert off == len(data)


def test_constant_input_codes_small_and_deterministic():
    w = h = 256
    nb = (w // 4) * (h // 4)
    final = np.full(nb, 0xAAAAAAAA_F800001F, np.uint64)
    motion = np.zeros(2 * nb, np.uint8)
    a = write_stream([(final, motion, np.zeros(0, np.uint32))] * 2, w, h, 8, 1)
    b = write_stream([(final, motion, np.zeros(0, np.uint32))] * 2, w, h, 8, 1)
    assert a == b
    assert len(a) < 34 + 2 * 2000


@pytest.mark.parametrize("w,h,sa,ui,n", [(255, 256, 8, 1, 1), (256, 320, 8, 1, 1), (256, 256, 0, 1, 1),
                                          (256, 256, 64, 1, 1), (256, 256, 8, 0, 1),
                                          (256, 256, 8, 256, 1), (256, 256, 8, 1, -1),
                                          (32768, 65536, 8, 1, 1)])  # above 2^30 pixels
def test_writer_rejects_bad_parameters(w, h, sa, ui, n):
    with pytest.raises(MptcError):
        StreamWriter(w, h, sa, ui, n)


def test_writer_rejects_mismatched_arrays():
    sw = StreamWriter(256, 256, 8, 1, 1)
    nb = 64 * 64
    with pytest.raises(ValueError):
        sw.add_frame(np.zeros(nb - 1, np.uint64), np.zeros(2 * nb, np.uint8), np.zeros(0, np.uint32))
    with pytest.raises(MptcError):
        sw.add_frame(np.zeros(nb, np.uint64), np.zeros(2 * nb, np.uint8), np.zeros(nb + 1, np.uint32))
    sw.close()


# ---- reader -------------------------------------------------------------------

def _oracle_stream(case):
    spec = StreamSpec(**case["spec"])
    frames = spec.generate(case["first"], case["count"])
    res = oracle.encode_stream(frames, case["search_area"], case["threshold"], case["intra_interval"],
                               threads=os.cpu_count() or 1, want_psnr=False)
    return spec, res, write_stream(res, spec.width, spec.height, case["search_area"],
                                   case["unique_interval"])


@pytest.mark.parametrize("case", STREAMS, ids=[c["name"] for c in STREAMS])
def test_reader_recovers_frames_and_rewrites_identical_stream(case):
    """Reader -> (motion, coefficients, palette) -> writer from coefficients
    reproduces the reference stream; motion codes and palettes are the
    encoder's (only complete groups are in the stream)."""
    from mptc_gb300.stream import StreamReader
    spec, res, data = _oracle_stream(case)
    assert hashlib.sha256(data).hexdigest() == case["sha"]
    rd = StreamReader(data)
    ui = case["unique_interval"]
    assert (rd.info.width, rd.info.height, rd.info.search_area, rd.info.unique_interval) == \
        (spec.width, spec.height, case["search_area"], ui)
    assert rd.info.frames == (case["count"] // ui) * ui
    sw = StreamWriter(spec.width, spec.height, case["search_area"], ui, case["count"])
    got = 0
    for k, (motion, coeff, unique) in enumerate(rd):
        np.testing.assert_array_equal(motion, res[k].motion)
        np.testing.assert_array_equal(unique, res[k].unique)
        sw.add_frame_coefficients(coeff, motion, unique)
        got += 1
    assert got == rd.info.frames
    # frames after the last complete group are coded but not written
    for r in res[got:]:
        sw.add_frame(r.final, r.motion, r.unique)
    assert hashlib.sha256(sw.finish()).hexdigest() == case["sha"]
    sw.close()
    rd.close()


def test_reader_rejects_truncated_and_bad_streams():
    from mptc_gb300.stream import StreamReader
    case = STREAMS[2]
    _, _, data = _oracle_stream(case)
    with pytest.raises(MptcError):
        StreamReader(data[:20])
    bad = bytearray(data)
    bad[9] = 0  # search area 0
    with pytest.raises(MptcError):
        StreamReader(bytes(bad))
    huge = bytearray(data)
    huge[0:8] = (65536).to_bytes(4, "little") + (32768).to_bytes(4, "little")  # 2^31 pixels
    with pytest.raises(MptcError):
        StreamReader(bytes(huge))
    rd = StreamReader(data[: len(data) // 2])
    with pytest.raises(MptcError):
        for _ in rd:
            pass
    rd.close()


def test_arithmetic_coder_round_trip_on_skewed_and_uniform_bytes():
    """Writer and reader coders are inverse on long runs, skewed and uniform
    symbol statistics (model rescaling, carries, renormalisation)."""
    from mptc_gb300.stream import StreamReader
    w = h = 256
    nb = (w // 4) * (h // 4)
    rng = np.random.default_rng(11)
    frames = []
    for k in range(3):
        motion = (rng.geometric(0.3 + 0.3 * k, 2 * nb) % 256).astype(np.uint8)
        if k == 2:
            motion = rng.integers(0, 256, 2 * nb, dtype=np.uint8)
        coeff = rng.integers(0, 256, 6 * nb, dtype=np.uint8) if k else np.full(6 * nb, 128, np.uint8)
        unique = rng.integers(0, 2**32, 17 * k, dtype=np.uint32)
        frames.append((motion, coeff, unique))
    sw = StreamWriter(w, h, 8, 1, 3)
    for m, c, u in frames:
        sw.add_frame_coefficients(c, m, u)
    data = sw.finish()
    sw.close()
    rd = StreamReader(data)
    for (m, c, u), (m2, c2, u2) in zip(frames, rd):
        np.testing.assert_array_equal(m, m2)
        np.testing.assert_array_equal(c, c2)
        np.testing.assert_array_equal(u, u2)
    rd.close()


def test_add_frames_matches_frame_by_frame_and_coefficients():
    """One add_frames call (frames coded on all host cores) writes the bytes of
    frame-by-frame add_frame calls, including a trailing partial group; the
    coefficient form, fed the planes the reader decodes, writes them again."""
    from mptc_gb300.stream import StreamReader
    w_, h_, nf, ui = 256, 512, 7, 3
    frames = StreamSpec(w_, h_, nf, seed=77, n_squares=3, square_size=48).generate()
    res = oracle.encode_stream(frames, 6, 5, 4, threads=os.cpu_count() or 1, want_psnr=False)
    one = StreamWriter(w_, h_, 6, ui, nf)
    for r in res:
        one.add_frame(r.final, r.motion, r.unique)
    ref = one.finish()
    one.close()
    n = (w_ // 4) * (h_ // 4)
    fin = np.stack([r.final for r in res])
    mot = np.stack([r.motion for r in res])
    nu = np.array([len(r.unique) for r in res], np.uint32)
    uni = np.zeros((nf, n), np.uint32)
    for k, r in enumerate(res):
        uni[k, : nu[k]] = r.unique
    run = StreamWriter(w_, h_, 6, ui, nf)
    run.add_frames(fin[:2], mot[:2], uni[:2], nu[:2])  # two calls: the group spans them
    run.add_frames(fin[2:], mot[2:], uni[2:], nu[2:])
    assert run.finish() == ref
    run.close()
    parts = list(StreamReader(ref))
    assert len(parts) == 6  # the trailing partial group is not written, as in the reference
    coeff = np.stack([p[1] for p in parts])
    cw = StreamWriter(w_, h_, 6, ui, 6)
    cw.add_frames(coeff, mot[:6], uni[:6], nu[:6], coefficients=True)
    data = cw.finish()
    cw.close()
    assert data == ref  # same group count (6 // 3 == 7 // 3) and the same records


def test_add_frames_chunk_boundaries_inside_one_call(monkeypatch):
    """With one host thread the writer codes runs in chunks of 2 frames, so one
    add_frames call of 7 frames crosses three chunk boundaries, two of them
    inside a unique group; the bytes equal frame-by-frame calls. write_stream
    in chunks of 2 and 5 frames writes them too."""
    from mptc_gb300.stream import write_stream
    w_, h_, nf, ui = 256, 256, 7, 3
    frames = StreamSpec(w_, h_, nf, seed=78, n_squares=2, square_size=40).generate()
    res = oracle.encode_stream(frames, 4, 5, 4, threads=os.cpu_count() or 1, want_psnr=False)
    one = StreamWriter(w_, h_, 4, ui, nf)
    for r in res:
        one.add_frame(r.final, r.motion, r.unique)
    ref = one.finish()
    one.close()
    n = (w_ // 4) * (h_ // 4)
    nu = np.array([len(r.unique) for r in res], np.uint32)
    uni = np.zeros((nf, n), np.uint32)
    for k, r in enumerate(res):
        uni[k, : nu[k]] = r.unique
    monkeypatch.setenv("MPTC_HOST_THREADS", "1")
    run = StreamWriter(w_, h_, 4, ui, nf)
    run.add_frames(np.stack([r.final for r in res]), np.stack([r.motion for r in res]), uni, nu)
    assert run.finish() == ref
    run.close()
    monkeypatch.delenv("MPTC_HOST_THREADS")
    for chunk in (2, 5):
        assert write_stream(res, w_, h_, 4, ui, chunk_frames=chunk) == ref


def test_add_frames_rejects_bad_runs():
    n = (256 // 4) * (256 // 4)
    w = StreamWriter(256, 256, 8, 2, 2)
    fin, mot = np.zeros((2, n), np.uint64), np.full((2, 2 * n), 255, np.uint8)
    uni = np.zeros((2, n), np.uint32)
    with pytest.raises(MptcError):  # a palette longer than the frame
        w.add_frames(fin, mot, uni, np.array([n + 1, 0], np.uint32))
    with pytest.raises(ValueError):  # one frame's motion codes for a run of two
        w.add_frames(fin, mot[:1], uni, np.array([0, 0], np.uint32))
    w.add_frames(fin, mot, uni, np.array([n, n], np.uint32))
    assert len(w.finish()) > 34
    w.close()


def test_reader_next_frames_matches_next_frame():
    """The reader's run call (parts of many frames decoded on all host cores)
    returns what frame-by-frame reads return, stops at the end of the stream,
    and rejects a truncated stream."""
    from mptc_gb300.stream import StreamReader
    case = STREAMS[2]
    _, _, data = _oracle_stream(case)
    one = list(StreamReader(data))
    rd = StreamReader(data)
    got = []
    while True:
        mot, coeff, uni, nu = rd.next_frames(3)
        if len(nu) == 0:
            break
        got += [(mot[f], coeff[f], uni[f, : nu[f]]) for f in range(len(nu))]
    rd.close()
    assert len(got) == len(one) > 3
    for a, b in zip(got, one):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
    rd = StreamReader(data[: len(data) // 2])
    with pytest.raises(MptcError):
        for _ in range(len(one)):
            rd.next_frames(len(one))
    rd.close()
