"""The oracle against the golden vectors recorded from the unmodified reference
encoder (DXTImage ctor + Reencode, codec/dxt_image.cpp:385-436, :868-957)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from mptc_gb300.synth import StreamSpec

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load_cases():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)["cases"]


CASES = load_cases()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_oracle_matches_reference_stream(case):
    spec = StreamSpec(**case["spec"])
    frames = spec.generate(case["first"], case["count"])
    # the generator is integer-exact: the inputs must be the reference's inputs
    assert [sha(f) for f in frames] == case["input_sha"]
    res = oracle.encode_stream(frames, case["search_area"], case["threshold"],
                               case["intra_interval"], threads=8)
    for k, (r, g) in enumerate(zip(res, case["frames"])):
        assert sha(r.stb) == g["stb"], f"frame {k}: stb blocks"
        assert sha(r.final) == g["final"], f"frame {k}: final blocks"
        assert sha(r.motion) == g["motion"], f"frame {k}: motion codes"
        assert sha(r.unique) == g["unique"], f"frame {k}: unique palette"
        assert r.stats.n_unique == g["n_unique"]
        assert r.stats.n_inter == g["n_inter"] and r.stats.n_intra == g["n_intra"]
        assert abs(r.psnr - g["psnr"]) <= 1e-9 * abs(g["psnr"])


@pytest.mark.parametrize("key", ["adv_sa4_thr5_ii16", "adv_sa2_thr0_ii1"])
def test_oracle_matches_reference_adversarial(key):
    z = np.load(os.path.join(GOLDEN, f"{key}.npz"))
    sa, thr, ii = (int(v) for v in z["params"])
    res = oracle.encode_stream(z["frames"], sa, thr, ii)
    np.testing.assert_array_equal(np.stack([r.stb for r in res]), z["stb"])
    np.testing.assert_array_equal(np.stack([r.final for r in res]), z["final"])
    np.testing.assert_array_equal(np.stack([r.motion for r in res]), z["motion"])
    np.testing.assert_array_equal(np.concatenate([r.unique for r in res]), z["unique"])
    np.testing.assert_allclose([r.psnr for r in res], z["psnr"], rtol=1e-12)


def test_oracle_threaded_equals_single_thread():
    frames = StreamSpec(128, 128, 3, seed=3).generate()
    a = oracle.encode_stream(frames, 8, 5, 16, threads=1)
    b = oracle.encode_stream(frames, 8, 5, 16, threads=5)
    for x, y in zip(a, b):
        assert np.array_equal(x.final, y.final) and np.array_equal(x.motion, y.motion)


def test_oracle_rejects_bad_sizes():
    with pytest.raises(ValueError):
        oracle.dxt1_encode(np.zeros((6, 8, 3), np.uint8))


def _decoded_sse_numpy(frame, blocks):
    """Plain numpy restatement: Decode565 (codec/dxt_image.cpp:43-61) and the
    PhysicalToLogical palette (:198-227) of every block, squared error."""
    h, w, _ = frame.shape
    b = blocks.astype(np.uint64)
    e = [(b >> np.uint64(s)) & np.uint64(0xFFFF) for s in (0, 16)]
    e = [x.astype(np.int64) for x in e]

    def dec(v):
        r, g, bl = v >> 11, (v >> 5) & 63, v & 31
        return np.stack([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (bl << 3) | (bl >> 2)], -1)
    c0, c1 = dec(e[0]), dec(e[1])
    four = (e[0] > e[1])[:, None]
    c2 = np.where(four, (2 * c0 + c1) // 3, (c0 + c1) // 2)
    c3 = np.where(four, (c0 + 2 * c1) // 3, 0)
    pal = np.stack([c0, c1, c2, c3], 1)  # (n, 4, 3)
    idx = np.stack([((b >> np.uint64(32 + 2 * i)) & np.uint64(3)).astype(np.int64) for i in range(16)], 1)
    px = frame.astype(np.int64).reshape(h // 4, 4, w // 4, 4, 3).transpose(0, 2, 1, 3, 4).reshape(-1, 16, 3)
    dec_px = np.take_along_axis(pal, idx[:, :, None].repeat(3, 2), 1)
    return int(((px - dec_px) ** 2).sum())


def test_oracle_decoded_sse():
    """The decoded-block squared error (the quantity the learned proposal's
    PSNR gate compares) equals a numpy restatement on an encoded stream, and on
    a frame where no block is accepted (every block keeps its stb block, so the
    logical palettes are PhysicalToLogical's) it gives the PSNR of the pinned
    DXTImage::PSNR restatement."""
    frames = StreamSpec(96, 64, 3, seed=31).generate()
    for r, f in zip(oracle.encode_stream(frames, 4, 5, 16, threads=4), frames):
        assert oracle.decoded_sse(f, r.final) == _decoded_sse_numpy(f, r.final)
        assert oracle.decoded_sse(f, r.stb) == _decoded_sse_numpy(f, r.stb)
    f = frames[1]
    stb = oracle.dxt1_encode(f)
    r = oracle.reencode(f, stb, None, 4, -(1 << 20))
    assert np.array_equal(r.final, stb)
    mse = oracle.decoded_sse(f, r.final) / (f.shape[0] * f.shape[1])
    assert abs(10.0 * np.log10(3.0 * 255.0 ** 2 / mse) - r.psnr) <= 1e-9 * r.psnr
