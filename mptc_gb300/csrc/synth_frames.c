/*
 * Seeded synthetic RGB8 video frames for the MPTC encoder workloads.
 *
 * The reference ships no sample video (the path codec/codec.cpp:406 points at
 * data that is not part of the project), so every workload is generated here:
 * per channel the sum of four low-frequency 2-D sinusoids around mid-grey,
 * plus square patches of uniform-noise texture that translate a few pixels per
 * frame, plus per-pixel uniform noise in [-4, 4], clamped to [0, 255].
 *
 * Everything is integer arithmetic (splitmix64 counters, a parabolic integer
 * sine, fixed-point positions), so the same seed yields the same bytes on any
 * host: the x86 build machine and the aarch64 GPU host agree bit for bit.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "synth_frames.h"

static uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Counter-based draw: value number `idx` of the stream named `tag`. */
static uint64_t draw(uint64_t seed, uint64_t tag, uint64_t idx) {
  return mix64(mix64(seed * 0xD1B54A32D192ED03ull + tag) ^ (idx * 0x9E3779B97F4A7C15ull));
}

static int draw_range(uint64_t seed, uint64_t tag, uint64_t idx, int lo, int hi) {
  uint64_t span = (uint64_t)(hi - lo + 1);
  return lo + (int)((draw(seed, tag, idx) >> 11) % span);
}

/* Parabolic integer sine: phase in [0, 2^32) is one full turn, result in
 * [-16384, 16384]. */
static int32_t isin(uint32_t phase) {
  int32_t h = (int32_t)((phase >> 16) & 0x7FFF);   /* position in the half turn */
  int32_t s = (int32_t)(((int64_t)h * (32768 - h)) >> 14);
  return (phase & 0x80000000u) ? -s : s;
}

static int32_t icos(uint32_t phase) { return isin(phase + 0x40000000u); }

static int floor_shift14(int64_t v) {  /* floor(v / 2^14) without relying on >> of negatives */
  return (int)(v >= 0 ? v / 16384 : -((-v + 16383) / 16384));
}

static int pos_mod(int64_t v, int m) {
  int64_t r = v % m;
  return (int)(r < 0 ? r + m : r);
}

enum { TAG_WAVE = 1, TAG_SQUARE = 2, TAG_TEXTURE = 3, TAG_NOISE = 4 };

typedef struct {
  int32_t amp;
  uint32_t phase0;
  int64_t kx, ky;  /* phase step per pixel, units of 2^-32 turns */
} wave_t;

static void make_waves(const mptc_synth_config *c, int segment, wave_t w[3][4]) {
  for (int ch = 0; ch < 3; ++ch) {
    for (int k = 0; k < 4; ++k) {
      uint64_t base = ((uint64_t)segment * 3 + ch) * 4 + k;
      uint64_t idx = base * 8;
      int period = draw_range(c->seed, TAG_WAVE, idx + 0, c->period_min, c->period_max);
      int amp = draw_range(c->seed, TAG_WAVE, idx + 1, c->amp_min, c->amp_max);
      uint32_t phase0 = (uint32_t)draw(c->seed, TAG_WAVE, idx + 2);
      uint32_t dir = (uint32_t)draw(c->seed, TAG_WAVE, idx + 3);
      w[ch][k].amp = amp;
      w[ch][k].phase0 = phase0;
      w[ch][k].kx = ((int64_t)icos(dir) << 18) / period;
      w[ch][k].ky = ((int64_t)isin(dir) << 18) / period;
    }
  }
}

int mptc_synth_frame(const mptc_synth_config *c, int frame, uint8_t *out) {
  if (!c || !out || c->width <= 0 || c->height <= 0 || frame < 0) return -1;
  if (c->period_min <= 0 || c->period_max < c->period_min) return -1;
  if (c->amp_max < c->amp_min || c->n_squares < 0 || c->square_size < 0) return -1;
  if (c->speed_max < c->speed_min) return -1;
  const int W = c->width, H = c->height;
  const int segment = c->cut_every > 0 ? frame / c->cut_every : 0;

  wave_t waves[3][4];
  make_waves(c, segment, waves);

  /* Background: four sinusoids per channel around 128. */
  for (int y = 0; y < H; ++y) {
    uint8_t *row = out + (size_t)y * W * 3;
    for (int ch = 0; ch < 3; ++ch) {
      uint32_t ph[4];
      for (int k = 0; k < 4; ++k)
        ph[k] = waves[ch][k].phase0 + (uint32_t)((int64_t)y * waves[ch][k].ky);
      for (int x = 0; x < W; ++x) {
        int v = 128;
        for (int k = 0; k < 4; ++k) {
          uint32_t p = ph[k] + (uint32_t)((int64_t)x * waves[ch][k].kx);
          v += floor_shift14((int64_t)waves[ch][k].amp * isin(p));
        }
        row[x * 3 + ch] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
      }
    }
  }

  /* Noise-textured squares translating at a seeded velocity (wrapping). */
  const int S = c->square_size;
  for (int q = 0; q < c->n_squares && S > 0; ++q) {
    uint64_t idx = (uint64_t)q * 8;
    int x0 = draw_range(c->seed, TAG_SQUARE, idx + 0, 0, W - 1);
    int y0 = draw_range(c->seed, TAG_SQUARE, idx + 1, 0, H - 1);
    int speed = draw_range(c->seed, TAG_SQUARE, idx + 2, c->speed_min, c->speed_max);
    uint32_t dir = (uint32_t)draw(c->seed, TAG_SQUARE, idx + 3);
    int64_t vx = ((int64_t)speed * icos(dir)) / 64;  /* 1/256 px per frame */
    int64_t vy = ((int64_t)speed * isin(dir)) / 64;
    int px = pos_mod(((int64_t)x0 * 256 + (int64_t)frame * vx) / 256, W);
    int py = pos_mod(((int64_t)y0 * 256 + (int64_t)frame * vy) / 256, H);
    for (int ty = 0; ty < S; ++ty) {
      int y = (py + ty) % H;
      for (int tx = 0; tx < S; ++tx) {
        int x = (px + tx) % W;
        uint64_t t = draw(c->seed, TAG_TEXTURE + 16 * (uint64_t)q, (uint64_t)ty * S + tx);
        uint8_t *p = out + ((size_t)y * W + x) * 3;
        p[0] = (uint8_t)(t & 0xFF);
        p[1] = (uint8_t)((t >> 8) & 0xFF);
        p[2] = (uint8_t)((t >> 16) & 0xFF);
      }
    }
  }

  /* Per-pixel uniform noise in [-4, 4]. */
  const uint64_t ntag = TAG_NOISE + 64 * (uint64_t)frame;
  const size_t n = (size_t)W * H * 3;
  for (size_t i = 0; i < n; ++i) {
    int v = out[i] + (int)((draw(c->seed, ntag, i) >> 32) % 9) - 4;
    out[i] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
  }
  return 0;
}

int mptc_synth_frames(const mptc_synth_config *c, int first, int count, uint8_t *out) {
  if (!c || count < 0) return -1;
  const size_t fsz = (size_t)c->width * c->height * 3;
  for (int f = 0; f < count; ++f) {
    int rc = mptc_synth_frame(c, first + f, out + fsz * f);
    if (rc) return rc;
  }
  return 0;
}
