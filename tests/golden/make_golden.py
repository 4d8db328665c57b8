"""Generate the golden vectors that pin the oracle to the reference encoder.

Runs the UNMODIFIED reference hot path (``DXTImage`` constructor +
``DXTImage::Reencode``, built from the reference sources by
``oracle/ref/Makefile`` into ``oracle/_ref/hotpath_harness``) on seeded
synthetic streams and on adversarial block patterns, and records:

* ``golden.json``      SHA-256 per frame of the stb blocks, final blocks,
                       motion codes and unique palette, plus PSNR, for each
                       case (inputs are regenerated from the integer-exact
                       synthetic generator, so only hashes are stored);
* ``adversarial.npz``  full input frames and outputs of the adversarial case;
* ``golden.json["streams"]``  SHA-256 and size of whole MPTC streams written
                       by the unmodified reference encoder (``CompressMultiUnique``
                       via ``oracle/_ref/mptc_encoder``, fed PNG frames), which
                       pin the host stream writer byte for byte, and SHA-256 per
                       frame of the blocks the unmodified reference decoder
                       (``GetFrame`` via ``oracle/_ref/decoder_harness``)
                       rebuilds from each stream, which pin the GPU decoder.

``configs.json`` (``--configs``) holds the same per-frame records for the
measured workloads at their full sizes: all 120 frames of the 1080p stream,
all 64 frames of the 720p stream with its scene cut (and its whole MPTC stream,
edge-padded to 1280x768), one stream of each resolution of the mixed batch,
and the 2160p stress stream at the largest search area (63); the reference
runs of these take most of an hour on one core each, so they run side by side.

Usage (needs the reference sources; run from the repository root):
    make -C oracle/ref REF=<path to MPTC>
    python tests/golden/make_golden.py            # golden.json + adversarial fixtures
    python tests/golden/make_golden.py --configs  # configs.json
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import struct
import tempfile
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from mptc_gb300.synth import (HD720, FHD1080, SMOKE_256, StreamSpec, mixed_batch, pad_edge,  # noqa: E402
                              uhd_streams)

HARNESS = os.path.join(ROOT, "oracle", "_ref", "hotpath_harness")
ENCODER = os.path.join(ROOT, "oracle", "_ref", "mptc_encoder")
DECODER = os.path.join(ROOT, "oracle", "_ref", "decoder_harness")
OUT_DIR = os.path.dirname(os.path.abspath(__file__))

# (name, spec, first frame, frame count, search_area, threshold, intra_interval)
CASES = [
    ("smoke256_sa8_thr5", SMOKE_256, 0, 16, 8, 5, 16),
    ("smoke256_sa4_thr0_ii4", SMOKE_256, 0, 8, 4, 0, 4),
    ("smoke256_sa16_thr20_ii8", SMOKE_256, 0, 4, 16, 20, 8),
    ("small64_sa1_thr5", StreamSpec(64, 64, 6, seed=7), 0, 6, 1, 5, 16),
    ("small128x96_sa2_thrm1", StreamSpec(128, 96, 5, seed=8), 0, 5, 2, -1, 2),
    ("small96x64_sa4_thr30_allintra", StreamSpec(96, 64, 6, seed=9), 0, 6, 4, 30, 1),
    ("small64_sa63_thr5", StreamSpec(64, 64, 4, seed=10), 0, 4, 63, 5, 2),
    ("small160x120_sa8_thr1000", StreamSpec(160, 120, 3, seed=11), 0, 3, 8, 1000, 2),
    ("small200x52_sa3_thr2", StreamSpec(200, 52, 5, seed=12, square_size=24), 0, 5, 3, 2, 3),
    ("hd720_cut_sa8_thr5", HD720, 30, 4, 8, 5, 16),
    ("fhd1080_sa8_thr5", FHD1080, 0, 2, 8, 5, 16),
]


# (name, spec, first frame, frame count, search_area, threshold, intra_interval,
#  unique_interval): whole streams; frame sizes are multiples of 256 pixels.
STREAM_CASES = [
    ("stream256_sa8_thr5_ii16_ui8", SMOKE_256, 0, 16, 8, 5, 16, 8),
    ("stream256_sa4_thr0_ii4_ui3_tail", SMOKE_256, 0, 8, 4, 0, 4, 3),
    ("stream512x256_sa2_thr20_ii2_ui1", StreamSpec(512, 256, 4, seed=21, n_squares=3), 0, 4, 2, 20, 2, 1),
    ("stream256x512_sa16_thr5_ii8_ui4", StreamSpec(256, 512, 8, seed=22, cut_every=3), 0, 8, 16, 5, 8, 4),
]


# The measured workloads at full size: (name, spec, first frame, frame count,
# search_area, threshold, intra_interval).
def config_cases():
    mixed = mixed_batch()
    return [
        ("fhd1080_120f_sa8_thr5", FHD1080, 0, 120, 8, 5, 16),
        ("hd720_64f_sa8_thr5", HD720, 0, 64, 8, 5, 16),
        ("mixed_856x480_s1000", mixed[0], 0, 4, 8, 5, 16),
        ("mixed_1280x720_s1009", mixed[9], 0, 4, 8, 5, 16),
        ("mixed_1920x1080_s1018", mixed[18], 0, 4, 8, 5, 16),
        ("mixed_2560x1440_s1027", mixed[27], 0, 4, 8, 5, 16),
        ("uhd2160_sa63_thr5", uhd_streams()[0], 0, 2, 63, 5, 16),
    ]


# Whole streams of the measured workloads, frames edge-padded to 256-pixel
# multiples: (name, spec, frame count, sa, thr, intra interval, unique interval).
CONFIG_STREAMS = [
    ("hd720_pad1280x768_64f_sa8_thr5_ii16_ui8", HD720, 64, 8, 5, 16, 8),
]


def adversarial_frames(n_frames: int = 4, size: int = 64, seed: int = 1234) -> np.ndarray:
    """Blocks that exercise stb_dxt's special cases and the refit edge cases:
    constant colours (incl. 0/255), two-colour splits, ramps, saturated
    channels, single outliers, near-constant blocks and pure noise. Later
    frames shift the pattern by whole blocks so that inter matches exist."""
    rng = np.random.default_rng(seed)
    nb = size // 4
    base = np.zeros((size, size, 3), np.uint8)
    kinds = 12
    for by in range(nb):
        for bx in range(nb):
            k = (by * nb + bx) % kinds
            blk = np.zeros((4, 4, 3), np.int32)
            c0 = rng.integers(0, 256, 3)
            c1 = rng.integers(0, 256, 3)
            if k == 0:
                blk[:] = c0
            elif k == 1:
                blk[:] = 0
            elif k == 2:
                blk[:] = 255
            elif k == 3:
                m = rng.integers(0, 2, (4, 4)).astype(bool)
                blk[m] = c0
                blk[~m] = c1
            elif k == 4:
                t = np.linspace(0, 1, 4)[None, :, None]
                blk[:] = (c0 * (1 - t) + c1 * t).round().astype(np.int32)
            elif k == 5:
                t = np.linspace(0, 1, 4)[:, None, None]
                blk[:] = (c0 * (1 - t) + c1 * t).round().astype(np.int32)
            elif k == 6:
                blk[..., 0] = 255
                blk[..., 1] = np.arange(16).reshape(4, 4) * 17
                blk[..., 2] = 0
            elif k == 7:
                blk[:] = c0
                blk[rng.integers(0, 4), rng.integers(0, 4)] = c1
            elif k == 8:
                blk[:] = c0
                blk += rng.integers(-1, 2, (4, 4, 3))
            elif k == 9:
                blk[:] = rng.integers(0, 256, (4, 4, 3))
            elif k == 10:
                g = np.arange(16).reshape(4, 4, 1) * 16
                blk[:] = g
            else:
                pal = rng.integers(0, 256, (4, 3))
                blk[:] = pal[rng.integers(0, 4, (4, 4))]
            base[4 * by:4 * by + 4, 4 * bx:4 * bx + 4] = np.clip(blk, 0, 255)
    frames = []
    for f in range(n_frames):
        fr = np.roll(base, shift=(4 * (f % 2), 4 * f), axis=(0, 1)).copy()
        if f >= 2:  # perturb a few blocks so that some searches fail
            fr[::8, ::8] = 255 - fr[::8, ::8]
        frames.append(fr)
    return np.stack(frames)


def run_reference(frames: np.ndarray, sa: int, thr: int, ii: int):
    n, h, w, _ = frames.shape
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "in.rgb")
        outp = os.path.join(td, "out.bin")
        np.ascontiguousarray(frames).tofile(inp)
        subprocess.check_call([HARNESS, inp, str(w), str(h), str(n), str(sa), str(thr), str(ii),
                               outp, td])
        buf = open(outp, "rb").read()
    nblk = (w // 4) * (h // 4)
    off = 0
    res = []
    for _ in range(n):
        stb = np.frombuffer(buf, np.uint64, nblk, off); off += 8 * nblk
        fin = np.frombuffer(buf, np.uint64, nblk, off); off += 8 * nblk
        mot = np.frombuffer(buf, np.uint8, 2 * nblk, off); off += 2 * nblk
        nu = int(np.frombuffer(buf, np.uint32, 1, off)[0]); off += 4
        uni = np.frombuffer(buf, np.uint32, nu, off); off += 4 * nu
        psnr = float(np.frombuffer(buf, np.float64, 1, off)[0]); off += 8
        res.append(dict(stb=stb, final=fin, motion=mot, unique=uni, psnr=psnr))
    assert off == len(buf)
    return res


def write_png(path: str, rgb: np.ndarray) -> None:
    """8-bit RGB PNG, filter 0 on every row (lossless; any decoder reads it back)."""
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data))

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def run_reference_stream(frames: np.ndarray, sa: int, thr: int, ii: int, ui: int) -> bytes:
    """Stream bytes of the reference encoder (codec/encoder.cpp main ->
    CompressMultiUnique) over PNG frames named in display order."""
    with tempfile.TemporaryDirectory() as td:
        fdir = os.path.join(td, "frames")
        os.makedirs(fdir)
        for i, f in enumerate(frames):
            write_png(os.path.join(fdir, f"frame{i:05d}.png"), np.ascontiguousarray(f))
        out = os.path.join(td, "stream.mptc")
        os.makedirs(os.path.join(td, "dec"))
        os.makedirs(os.path.join(td, "ep"))
        subprocess.check_call([ENCODER, str(sa), str(ii), str(ui), str(thr), "1", fdir, out,
                               os.path.join(td, "dec"), os.path.join(td, "ep")],
                              cwd=td, stdout=subprocess.DEVNULL)
        return open(out, "rb").read()


def run_reference_decoder(data: bytes, n_frames: int) -> list[np.ndarray]:
    """Physical blocks of the first n_frames frames as the reference decoder's
    GetFrame (codec/decoder.cpp:256-414) rebuilds them."""
    h, w = struct.unpack_from("<II", data, 0)
    nblk = (w // 4) * (h // 4)
    with tempfile.TemporaryDirectory() as td:
        sp = os.path.join(td, "stream.mptc")
        op = os.path.join(td, "blocks.bin")
        open(sp, "wb").write(data)
        subprocess.check_call([DECODER, sp, str(n_frames), op], cwd=td, stdout=subprocess.DEVNULL)
        raw = np.fromfile(op, np.uint64)
    return list(raw.reshape(n_frames, nblk))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def frame_record(r) -> dict:
    mot = r["motion"].reshape(-1, 2)
    kinds = np.where((mot[:, 0] == 255) & (mot[:, 1] == 255), 0,
                     np.where(mot[:, 0] & 0x80, 2, 1))
    return dict(stb=sha(r["stb"]), final=sha(r["final"]), motion=sha(r["motion"]),
                unique=sha(r["unique"]), n_unique=int(r["unique"].size),
                n_inter=int((kinds == 2).sum()), n_intra=int((kinds == 1).sum()),
                psnr=r["psnr"])


def main() -> None:
    if not os.path.exists(HARNESS):
        sys.exit(f"{HARNESS} missing: build it with make -C oracle/ref")
    golden = {"generator": "mptc_gb300/csrc/synth_frames.c", "cases": []}
    for name, spec, first, count, sa, thr, ii in CASES:
        frames = spec.generate(first, count)
        res = run_reference(frames, sa, thr, ii)
        golden["cases"].append(dict(
            name=name, spec=spec.__dict__, first=first, count=count, search_area=sa,
            threshold=thr, intra_interval=ii, input_sha=[sha(f) for f in frames],
            frames=[frame_record(r) for r in res]))
        print(name, [(fr["n_inter"], fr["n_intra"], fr["n_unique"]) for fr in golden["cases"][-1]["frames"]])
    adv = adversarial_frames()
    for sa, thr, ii in [(4, 5, 16), (2, 0, 1)]:
        res = run_reference(adv, sa, thr, ii)
        key = f"adv_sa{sa}_thr{thr}_ii{ii}"
        np.savez_compressed(os.path.join(OUT_DIR, f"{key}.npz"), frames=adv,
                            stb=np.stack([r["stb"] for r in res]),
                            final=np.stack([r["final"] for r in res]),
                            motion=np.stack([r["motion"] for r in res]),
                            unique=np.concatenate([r["unique"] for r in res]),
                            n_unique=np.array([r["unique"].size for r in res]),
                            psnr=np.array([r["psnr"] for r in res]),
                            params=np.array([sa, thr, ii]))
        print(key, [r["unique"].size for r in res])
    golden["streams"] = []
    for name, spec, first, count, sa, thr, ii, ui in STREAM_CASES:
        frames = spec.generate(first, count)
        data = run_reference_stream(frames, sa, thr, ii, ui)
        # GetFrame rewinds after the first frame of the last group
        groups = count // ui
        n_dec = (groups - 1) * ui + 1
        decoded = run_reference_decoder(data, n_dec)
        golden["streams"].append(dict(
            name=name, spec=spec.__dict__, first=first, count=count, search_area=sa,
            threshold=thr, intra_interval=ii, unique_interval=ui,
            input_sha=[sha(f) for f in frames], size=len(data),
            sha=hashlib.sha256(data).hexdigest(), header=data[:34].hex(),
            decoded=[sha(b) for b in decoded]))
        print(name, len(data), "decoded", n_dec)
    with open(os.path.join(OUT_DIR, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)


def _config_case(case):
    name, spec, first, count, sa, thr, ii = case
    frames = spec.generate(first, count)
    res = run_reference(frames, sa, thr, ii)
    return dict(name=name, spec=spec.__dict__, first=first, count=count, search_area=sa,
                threshold=thr, intra_interval=ii, input_sha=[sha(f) for f in frames],
                frames=[frame_record(r) for r in res])


def _config_stream(case):
    name, spec, count, sa, thr, ii, ui = case
    frames = pad_edge(spec.generate(0, count), 256)
    data = run_reference_stream(frames, sa, thr, ii, ui)
    n_dec = (count // ui - 1) * ui + 1
    decoded = run_reference_decoder(data, n_dec)
    return dict(name=name, spec=spec.__dict__, count=count, pad=256, search_area=sa, threshold=thr,
                intra_interval=ii, unique_interval=ui, width=int(frames.shape[2]),
                height=int(frames.shape[1]), input_sha=[sha(f) for f in frames], size=len(data),
                sha=hashlib.sha256(data).hexdigest(), decoded=[sha(b) for b in decoded])


def main_configs() -> None:
    import multiprocessing as mp
    if not os.path.exists(HARNESS):
        sys.exit(f"{HARNESS} missing: build it with make -C oracle/ref")
    cases = config_cases()
    # longest first, so that the pool's last worker is not the slowest case
    order = sorted(range(len(cases)), key=lambda i: -cases[i][3] * cases[i][1].width * cases[i][1].height
                   * cases[i][4] ** 2)
    with mp.get_context("spawn").Pool(min(len(cases) + 1, os.cpu_count() or 1)) as pool:
        streams = [pool.apply_async(_config_stream, (c,)) for c in CONFIG_STREAMS]
        jobs = {i: pool.apply_async(_config_case, (cases[i],)) for i in order}
        out = {"generator": "mptc_gb300/csrc/synth_frames.c",
               "cases": [jobs[i].get() for i in range(len(cases))],
               "streams": [j.get() for j in streams]}
    for c in out["cases"]:
        print(c["name"], [(fr["n_inter"], fr["n_intra"], fr["n_unique"]) for fr in c["frames"]][:4])
    with open(os.path.join(OUT_DIR, "configs.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    if "--configs" in sys.argv[1:]:
        main_configs()
    else:
        main()
