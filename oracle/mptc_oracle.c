/*
 * ORACLE — test infrastructure only (see mptc_oracle.h).
 *
 * CPU restatement of the MPTC encoder hot path. Reference files cited below
 * are paths inside the MPTC project:
 *   Include/stb_dxt.h      stb_dxt v1.04 DXT1 encoder
 *   codec/dxt_image.cpp    DXTImage, CompressedBlock, IntraSearch, InterBlockSearch, Reencode
 *
 * Floating-point steps keep the reference's operation order; build with
 * -ffp-contract=off (no fused multiply-add) so x86-64 and aarch64 agree. The
 * reference's float->int casts are x86 cvttss2si, which yields INT_MIN for NaN
 * or out-of-range inputs; x86_cvtt() restates that explicitly.
 */
#include "mptc_oracle.h"

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* stb_dxt tables and helpers                                                */
/* ------------------------------------------------------------------------- */

static unsigned char g_expand5[32], g_expand6[64];
static unsigned char g_omatch5[256][2], g_omatch6[256][2];
static pthread_once_t g_tables_once = PTHREAD_ONCE_INIT;

/* stb__Mul8Bit, Include/stb_dxt.h:64-68 */
static int mul8bit(int a, int b) {
  int t = a * b + 128;
  return (t + (t >> 8)) >> 8;
}

/* stb__Lerp13 without rounding bias, Include/stb_dxt.h:88-98 */
static int lerp13(int a, int b) { return (2 * a + b) / 3; }

/* stb__PrepareOptTable, Include/stb_dxt.h:111-137 */
static void prepare_opt_table(unsigned char table[256][2], const unsigned char *expand, int size) {
  for (int i = 0; i < 256; i++) {
    int best = 256;
    for (int mn = 0; mn < size; mn++) {
      for (int mx = 0; mx < size; mx++) {
        int mine = expand[mn], maxe = expand[mx];
        int err = abs(lerp13(maxe, mine) - i);
        err += abs(maxe - mine) * 3 / 100;
        if (err < best) {
          table[i][0] = (unsigned char)mx;
          table[i][1] = (unsigned char)mn;
          best = err;
        }
      }
    }
  }
}

/* stb__InitDXT, Include/stb_dxt.h:593-611 (the dither tables are unused: mode has no DITHER bit) */
static void init_tables(void) {
  for (int i = 0; i < 32; i++) g_expand5[i] = (unsigned char)((i << 3) | (i >> 2));
  for (int i = 0; i < 64; i++) g_expand6[i] = (unsigned char)((i << 2) | (i >> 4));
  prepare_opt_table(g_omatch5, g_expand5, 32);
  prepare_opt_table(g_omatch6, g_expand6, 64);
}

/* stb__From16Bit, Include/stb_dxt.h:70-80 */
static void from16bit(unsigned char out[4], unsigned short v) {
  out[0] = g_expand5[(v & 0xf800) >> 11];
  out[1] = g_expand6[(v & 0x07e0) >> 5];
  out[2] = g_expand5[v & 0x001f];
  out[3] = 0;
}

/* stb__As16Bit, Include/stb_dxt.h:82-85 */
static unsigned short as16bit(int r, int g, int b) {
  return (unsigned short)((mul8bit(r, 31) << 11) + (mul8bit(g, 63) << 5) + mul8bit(b, 31));
}

/* stb__EvalColors, Include/stb_dxt.h:139-145 */
static void eval_colors(unsigned char color[16], unsigned short c0, unsigned short c1) {
  from16bit(color + 0, c0);
  from16bit(color + 4, c1);
  for (int k = 0; k < 3; k++) {
    color[8 + k] = (unsigned char)lerp13(color[0 + k], color[4 + k]);
    color[12 + k] = (unsigned char)lerp13(color[4 + k], color[0 + k]);
  }
}

/* stb__MatchColorsBlock, no-dither branch, Include/stb_dxt.h:176-215 */
static unsigned int match_colors(const unsigned char *block, const unsigned char *color) {
  unsigned int mask = 0;
  int dirr = color[0] - color[4];
  int dirg = color[1] - color[5];
  int dirb = color[2] - color[6];
  int dots[16], stops[4];
  for (int i = 0; i < 16; i++)
    dots[i] = block[i * 4 + 0] * dirr + block[i * 4 + 1] * dirg + block[i * 4 + 2] * dirb;
  for (int i = 0; i < 4; i++)
    stops[i] = color[i * 4 + 0] * dirr + color[i * 4 + 1] * dirg + color[i * 4 + 2] * dirb;
  int c0p = (stops[1] + stops[3]) >> 1;
  int halfp = (stops[3] + stops[2]) >> 1;
  int c3p = (stops[2] + stops[0]) >> 1;
  for (int i = 15; i >= 0; i--) {
    int dot = dots[i];
    mask <<= 2;
    if (dot < halfp)
      mask |= (dot < c0p) ? 1 : 3;
    else
      mask |= (dot < c3p) ? 2 : 0;
  }
  return mask;
}

/* stb__OptimizeColorsBlock, Include/stb_dxt.h:273-375 */
static void optimize_colors(const unsigned char *block, unsigned short *pmax16,
                            unsigned short *pmin16) {
  int mind = 0x7fffffff, maxd = -0x7fffffff;
  const unsigned char *minp = block, *maxp = block;
  int mu[3], mn[3], mx[3];
  for (int ch = 0; ch < 3; ch++) {
    const unsigned char *bp = block + ch;
    int muv = bp[0], minv = bp[0], maxv = bp[0];
    for (int i = 4; i < 64; i += 4) {
      muv += bp[i];
      if (bp[i] < minv)
        minv = bp[i];
      else if (bp[i] > maxv)
        maxv = bp[i];
    }
    mu[ch] = (muv + 8) >> 4;
    mn[ch] = minv;
    mx[ch] = maxv;
  }
  int cov[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 16; i++) {
    int r = block[i * 4 + 0] - mu[0];
    int g = block[i * 4 + 1] - mu[1];
    int b = block[i * 4 + 2] - mu[2];
    cov[0] += r * r;
    cov[1] += r * g;
    cov[2] += r * b;
    cov[3] += g * g;
    cov[4] += g * b;
    cov[5] += b * b;
  }
  float covf[6];
  for (int i = 0; i < 6; i++) covf[i] = (float)cov[i] / 255.0f;
  float vfr = (float)(mx[0] - mn[0]);
  float vfg = (float)(mx[1] - mn[1]);
  float vfb = (float)(mx[2] - mn[2]);
  for (int iter = 0; iter < 4; iter++) {
    float r = vfr * covf[0] + vfg * covf[1] + vfb * covf[2];
    float g = vfr * covf[1] + vfg * covf[3] + vfb * covf[4];
    float b = vfr * covf[2] + vfg * covf[4] + vfb * covf[5];
    vfr = r;
    vfg = g;
    vfb = b;
  }
  double magn = fabs(vfr);
  if (fabs(vfg) > magn) magn = fabs(vfg);
  if (fabs(vfb) > magn) magn = fabs(vfb);
  int v_r, v_g, v_b;
  if (magn < 4.0f) {
    v_r = 299;
    v_g = 587;
    v_b = 114;
  } else {
    magn = 512.0 / magn;
    v_r = (int)(vfr * magn);
    v_g = (int)(vfg * magn);
    v_b = (int)(vfb * magn);
  }
  for (int i = 0; i < 16; i++) {
    int dot = block[i * 4 + 0] * v_r + block[i * 4 + 1] * v_g + block[i * 4 + 2] * v_b;
    if (dot < mind) {
      mind = dot;
      minp = block + i * 4;
    }
    if (dot > maxd) {
      maxd = dot;
      maxp = block + i * 4;
    }
  }
  *pmax16 = as16bit(maxp[0], maxp[1], maxp[2]);
  *pmin16 = as16bit(minp[0], minp[1], minp[2]);
}

/* stb__sclamp, Include/stb_dxt.h:377-383 (the argument is always in int range here) */
static int sclamp(float y, int p0, int p1) {
  int x = (int)y;
  if (x < p0) return p0;
  if (x > p1) return p1;
  return x;
}

/* stb__RefineBlock, Include/stb_dxt.h:388-464 */
static int refine_block(const unsigned char *block, unsigned short *pmax16, unsigned short *pmin16,
                        unsigned int mask) {
  static const int w1tab[4] = {3, 0, 2, 1};
  static const int prods[4] = {0x090000, 0x000900, 0x040102, 0x010402};
  unsigned short old_min = *pmin16, old_max = *pmax16, min16, max16;
  if ((mask ^ (mask << 2)) < 4) {
    int r = 8, g = 8, b = 8;
    for (int i = 0; i < 16; ++i) {
      r += block[i * 4 + 0];
      g += block[i * 4 + 1];
      b += block[i * 4 + 2];
    }
    r >>= 4;
    g >>= 4;
    b >>= 4;
    max16 = (unsigned short)((g_omatch5[r][0] << 11) | (g_omatch6[g][0] << 5) | g_omatch5[b][0]);
    min16 = (unsigned short)((g_omatch5[r][1] << 11) | (g_omatch6[g][1] << 5) | g_omatch5[b][1]);
  } else {
    int akku = 0;
    int at1_r = 0, at1_g = 0, at1_b = 0, at2_r = 0, at2_g = 0, at2_b = 0;
    unsigned int cm = mask;
    for (int i = 0; i < 16; ++i, cm >>= 2) {
      int step = cm & 3;
      int w1 = w1tab[step];
      int r = block[i * 4 + 0], g = block[i * 4 + 1], b = block[i * 4 + 2];
      akku += prods[step];
      at1_r += w1 * r;
      at1_g += w1 * g;
      at1_b += w1 * b;
      at2_r += r;
      at2_g += g;
      at2_b += b;
    }
    at2_r = 3 * at2_r - at1_r;
    at2_g = 3 * at2_g - at1_g;
    at2_b = 3 * at2_b - at1_b;
    int xx = akku >> 16;
    int yy = (akku >> 8) & 0xff;
    int xy = (akku >> 0) & 0xff;
    float frb = 3.0f * 31.0f / 255.0f / (float)(xx * yy - xy * xy);
    float fg = frb * 63.0f / 31.0f;
    max16 = (unsigned short)(sclamp((float)(at1_r * yy - at2_r * xy) * frb + 0.5f, 0, 31) << 11);
    max16 |= (unsigned short)(sclamp((float)(at1_g * yy - at2_g * xy) * fg + 0.5f, 0, 63) << 5);
    max16 |= (unsigned short)(sclamp((float)(at1_b * yy - at2_b * xy) * frb + 0.5f, 0, 31) << 0);
    min16 = (unsigned short)(sclamp((float)(at2_r * xx - at1_r * xy) * frb + 0.5f, 0, 31) << 11);
    min16 |= (unsigned short)(sclamp((float)(at2_g * xx - at1_g * xy) * fg + 0.5f, 0, 63) << 5);
    min16 |= (unsigned short)(sclamp((float)(at2_b * xx - at1_b * xy) * frb + 0.5f, 0, 31) << 0);
  }
  *pmin16 = min16;
  *pmax16 = max16;
  return old_min != min16 || old_max != max16;
}

/* stb_compress_dxt_block(dest, src, alpha=0, STB_DXT_HIGHQUAL) ->
 * stb__CompressColorBlock, Include/stb_dxt.h:467-538 and :613-627 */
uint64_t mo_stb_encode_block(const uint8_t rgba[64]) {
  pthread_once(&g_tables_once, init_tables);
  const unsigned char *block = rgba;
  unsigned int mask;
  unsigned short max16, min16;
  unsigned char color[16];
  int i;
  for (i = 1; i < 16; i++)
    if (memcmp(block + 4 * i, block, 4) != 0) break;
  if (i == 16) {
    int r = block[0], g = block[1], b = block[2];
    mask = 0xaaaaaaaau;
    max16 = (unsigned short)((g_omatch5[r][0] << 11) | (g_omatch6[g][0] << 5) | g_omatch5[b][0]);
    min16 = (unsigned short)((g_omatch5[r][1] << 11) | (g_omatch6[g][1] << 5) | g_omatch5[b][1]);
  } else {
    optimize_colors(block, &max16, &min16);
    if (max16 != min16) {
      eval_colors(color, max16, min16);
      mask = match_colors(block, color);
    } else {
      mask = 0;
    }
    for (i = 0; i < 2; i++) {
      unsigned int lastmask = mask;
      if (refine_block(block, &max16, &min16, mask)) {
        if (max16 != min16) {
          eval_colors(color, max16, min16);
          mask = match_colors(block, color);
        } else {
          mask = 0;
          break;
        }
      }
      if (mask == lastmask) break;
    }
  }
  if (max16 < min16) {
    unsigned short t = min16;
    min16 = max16;
    max16 = t;
    mask ^= 0x55555555u;
  }
  return (uint64_t)max16 | ((uint64_t)min16 << 16) | ((uint64_t)mask << 32);
}

/* Frame driver: CompressRGB codec/dxt_image.cpp:123-149, loop :419-431 */
int mo_dxt1_encode_frame(const uint8_t *rgb, int width, int height, uint64_t *blocks) {
  if (!rgb || !blocks || width <= 0 || height <= 0 || (width & 3) || (height & 3)) return -1;
  const int bw = width >> 2, bh = height >> 2;
  uint8_t rgba[64];
  for (int by = 0; by < bh; ++by) {
    for (int bx = 0; bx < bw; ++bx) {
      for (int j = 0; j < 4; ++j) {
        for (int i = 0; i < 4; ++i) {
          const uint8_t *p = rgb + ((size_t)(4 * by + j) * width + 4 * bx + i) * 3;
          uint8_t *q = rgba + (j * 4 + i) * 4;
          q[0] = p[0];
          q[1] = p[1];
          q[2] = p[2];
          q[3] = 0xFF;
        }
      }
      blocks[(size_t)by * bw + bx] = mo_stb_encode_block(rgba);
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Logical blocks, refit and error (codec/dxt_image.cpp)                      */
/* ------------------------------------------------------------------------- */

/* Decode565, codec/dxt_image.cpp:43-61 */
static void decode565(uint16_t x, uint8_t out[3]) {
  uint32_t r = x >> 11, g = (x >> 5) & 0x3F, b = x & 0x1F;
  out[0] = (uint8_t)((r << 3) | (r >> 2));
  out[1] = (uint8_t)((g << 2) | (g >> 4));
  out[2] = (uint8_t)((b << 3) | (b >> 2));
}

/* Pack565, codec/dxt_image.cpp:63-69 */
static uint16_t pack565(const uint8_t in[3]) {
  return (uint16_t)(((in[0] & 0xF8) << 8) | ((in[1] & 0xFC) << 3) | ((in[2] & 0xF8) >> 3));
}

static uint8_t absdiff_u8(uint8_t a, uint8_t b) { return (uint8_t)(a > b ? a - b : b - a); }

/* ToFiveBits, codec/dxt_image.cpp:72-95 (reproduced with its +-4 neighbours) */
static uint8_t to_five_bits(uint8_t x) {
  uint8_t base = x & 0xF8;
  uint8_t high = base == 255 ? base : (uint8_t)(base + 0x4);
  uint8_t low = base == 0 ? base : (uint8_t)(base - 0x4);
  base = (uint8_t)(base | (base >> 5));
  high = (uint8_t)(high | (high >> 5));
  low = (uint8_t)(low | (low >> 5));
  uint8_t db = absdiff_u8(x, base), dh = absdiff_u8(x, high), dl = absdiff_u8(x, low);
  if (db <= dh) return db < dl ? base : low;
  return high;
}

/* ToSixBits, codec/dxt_image.cpp:98-121 */
static uint8_t to_six_bits(uint8_t x) {
  uint8_t base = x & 0xFC;
  uint8_t high = base == 255 ? base : (uint8_t)(base + 0x2);
  uint8_t low = base == 0 ? base : (uint8_t)(base - 0x2);
  base = (uint8_t)(base | (base >> 6));
  high = (uint8_t)(high | (high >> 6));
  low = (uint8_t)(low | (low >> 6));
  uint8_t db = absdiff_u8(x, base), dh = absdiff_u8(x, high), dl = absdiff_u8(x, low);
  if (db <= dh) return db < dl ? base : low;
  return high;
}

/* x86-64 cvttss2si: truncation, INT_MIN for NaN or results outside int32. */
static int32_t x86_cvtt(float v) {
  if (!(v > -2147483904.0f && v < 2147483648.0f)) return INT32_MIN;
  return (int32_t)v;
}

/* Palette of a physical block: PhysicalToLogical, codec/dxt_image.cpp:198-227,
 * with LerpChannels :34-41. Colour 3 of a 3-colour block is black. */
static void block_palette(uint64_t block, uint8_t pal[4][3]) {
  uint16_t e1 = (uint16_t)(block & 0xFFFF), e2 = (uint16_t)((block >> 16) & 0xFFFF);
  decode565(e1, pal[0]);
  decode565(e2, pal[1]);
  for (int c = 0; c < 3; ++c) {
    if (e1 <= e2) {
      pal[2][c] = (uint8_t)((pal[0][c] + pal[1][c]) / 2);
      pal[3][c] = 0;
    } else {
      pal[2][c] = (uint8_t)((pal[0][c] * 2 + pal[1][c]) / 3);
      pal[3][c] = (uint8_t)((pal[0][c] + pal[1][c] * 2) / 3);
    }
  }
}

/* CompressedBlock::Error, codec/dxt_image.cpp:258-276 */
static int palette_error(const uint8_t px[48], uint32_t interp, const uint8_t pal[4][3]) {
  uint32_t err = 0;
  for (int i = 0; i < 16; ++i) {
    int k = (interp >> (2 * i)) & 3;
    for (int c = 0; c < 3; ++c) {
      int d = (int)px[i * 3 + c] - (int)pal[k][c];
      err += (uint32_t)(d * d);
    }
  }
  return (int)(err / 48);
}

int mo_block_error(const uint8_t px[48], uint64_t block) {
  uint8_t pal[4][3];
  block_palette(block, pal);
  return palette_error(px, (uint32_t)(block >> 32), pal);
}

/* CompressedBlock::RecalculateEndpoints, codec/dxt_image.cpp:290-351 */
static void refit_endpoints(const uint8_t px[48], uint32_t interp, uint8_t ep1[3], uint8_t ep2[3]) {
  static const float idx_to_order[4] = {0.f, 3.f, 1.f, 2.f};
  float asq = 0.0f, bsq = 0.0f, ab = 0.0f;
  float ax[3] = {0.0f, 0.0f, 0.0f}, bx[3] = {0.0f, 0.0f, 0.0f};
  for (int i = 0; i < 16; i++) {
    const float order = idx_to_order[(interp >> (2 * i)) & 3];
    const float a = (3.0f - order) / 3.0f;
    const float b = order / 3.0f;
    asq += a * a;
    bsq += b * b;
    ab += a * b;
    for (int j = 0; j < 3; ++j) {
      ax[j] += (float)px[i * 3 + j] * a;
      bx[j] += (float)px[i * 3 + j] * b;
    }
  }
  float f = 1.0f / (asq * bsq - ab * ab);
  for (int c = 0; c < 3; ++c) {
    float p1 = f * (ax[c] * bsq - bx[c] * ab);
    float p2 = f * (bx[c] * asq - ax[c] * ab);
    int32_t q1 = x86_cvtt(p1 + 0.5f), q2 = x86_cvtt(p2 + 0.5f);
    q1 = q1 < 255 ? q1 : 255;
    q2 = q2 < 255 ? q2 : 255;
    ep1[c] = (uint8_t)(q1 > 0 ? q1 : 0);
    ep2[c] = (uint8_t)(q2 > 0 ? q2 : 0);
  }
  ep1[0] = to_five_bits(ep1[0]);
  ep2[0] = to_five_bits(ep2[0]);
  ep1[1] = to_six_bits(ep1[1]);
  ep2[1] = to_six_bits(ep2[1]);
  ep1[2] = to_five_bits(ep1[2]);
  ep2[2] = to_five_bits(ep2[2]);
}

/* Refit palette, codec/dxt_image.cpp:343-347 (always the 4-colour form). */
static void refit_palette(const uint8_t ep1[3], const uint8_t ep2[3], uint8_t pal[4][3]) {
  for (int c = 0; c < 3; ++c) {
    pal[0][c] = ep1[c];
    pal[1][c] = ep2[c];
    pal[2][c] = (uint8_t)((ep1[c] * 2 + ep2[c]) / 3);
    pal[3][c] = (uint8_t)((ep1[c] + ep2[c] * 2) / 3);
  }
}

int mo_refit(const uint8_t px[48], uint32_t interp, uint8_t ep1[3], uint8_t ep2[3], int *valid) {
  uint8_t pal[4][3];
  refit_endpoints(px, interp, ep1, ep2);
  refit_palette(ep1, ep2, pal);
  /* The refit keeps the candidate's indices only when LogicalToPhysical needs
   * no swap, i.e. Pack565(ep1) > Pack565(ep2) (codec/dxt_image.cpp:154-161,
   * :689-694); the refit palette's alpha is always 0xFF. */
  if (valid) *valid = pack565(ep1) > pack565(ep2);
  return palette_error(px, interp, pal);
}

/* ------------------------------------------------------------------------- */
/* Index-block search (codec/dxt_image.cpp:652-774) and Reencode (:868-957)   */
/* ------------------------------------------------------------------------- */

typedef struct {
  uint8_t px[48];
  uint64_t stb;
  int orig_err;
} block_ctx;

typedef struct {
  int min_err;     /* value returned by the search */
  int mx, my;      /* motion code components before the inter 0x80 flag */
  uint32_t interp; /* selected candidate */
  int refit;       /* re_assigned */
  int found;       /* at least one update happened */
} search_result;

/* Get4X4ColorsBlock, codec/dxt_image.cpp:636-650 */
static void gather_block(const uint8_t *rgb, int width, int bx, int by, uint8_t px[48]) {
  for (int row = 0; row < 4; ++row)
    memcpy(px + 12 * row, rgb + ((size_t)(4 * by + row) * width + 4 * bx) * 3, 12);
}

/* Evaluate one candidate: returns 0 when skipped (refit would swap), else 1
 * with *err = Error() of the candidate block and *refit = re_assigned.
 * Body of the candidate loops, codec/dxt_image.cpp:677-697 and :734-757. */
static int eval_candidate(const block_ctx *b, uint32_t cand, int *err, int *refit) {
  if (cand == (uint32_t)(b->stb >> 32)) { /* blk == blk2: AssignIndices was the identity */
    *err = b->orig_err;
    *refit = 0;
    return 1;
  }
  uint8_t ep1[3], ep2[3];
  int valid;
  int e = mo_refit(b->px, cand, ep1, ep2, &valid);
  if (!valid) return 0;
  *err = e;
  *refit = 1;
  return 1;
}

/* Shared update rule of both searches: strict improvement, and the first
 * candidate with err_diff <= 0 pins min_err to 0 and leaves the column loop
 * only (codec/dxt_image.cpp:698-708, :758-768). Returns 1 to break. */
static int update(search_result *r, int err_diff, int mx, int my, uint32_t cand, int refit) {
  if (err_diff < r->min_err) {
    r->min_err = err_diff;
    r->mx = mx;
    r->my = my;
    r->interp = cand;
    r->refit = refit;
    r->found = 1;
    if (err_diff <= 0) {
      r->min_err = 0;
      return 1;
    }
  }
  return 0;
}

/* InterBlockSearch, codec/dxt_image.cpp:715-774 */
static search_result inter_search(const block_ctx *b, int bx, int by, int bw, int bh, int sa,
                                  const uint64_t *prev_final, int64_t *visited, int64_t *refits) {
  search_result r = {INT_MAX, 0, 0, 0, 0, 0};
  for (int j = by - sa; j < by + sa; j++) {
    for (int i = bx - sa; i < bx + sa; i++) {
      if (i >= bw || j >= bh || j < 0 || i < 0) continue;
      uint32_t cand = (uint32_t)(prev_final[(size_t)j * bw + i] >> 32);
      int err, refit;
      ++*visited;
      int ok = eval_candidate(b, cand, &err, &refit);
      *refits += cand != (uint32_t)(b->stb >> 32);
      if (!ok) continue;
      if (update(&r, err - b->orig_err, (i - bx) + sa, (j - by) + sa, cand, refit)) break;
    }
  }
  return r;
}

/* IntraSearch, codec/dxt_image.cpp:652-713 (causal window over this frame's
 * blocks as finalised so far) */
static search_result intra_search(const block_ctx *b, int bx, int by, int bw, int bh, int sa,
                                  const uint64_t *cur_final, int64_t *visited, int64_t *refits) {
  search_result r = {INT_MAX, 0, 0, 0, 0, 0};
  for (int j = by; j >= by - 2 * sa + 1; j--) {
    for (int i = bx + (sa - 1); i >= bx - sa; i--) {
      if ((i >= bw || j >= bh || j < 0 || i < 0) || (j == by && i >= bx)) continue;
      uint32_t cand = (uint32_t)(cur_final[(size_t)j * bw + i] >> 32);
      int err, refit;
      ++*visited;
      int ok = eval_candidate(b, cand, &err, &refit);
      *refits += cand != (uint32_t)(b->stb >> 32);
      if (!ok) continue;
      if (update(&r, err - b->orig_err, (i - bx) + sa, (j - by) + 2 * sa - 1, cand, refit)) break;
    }
  }
  return r;
}

/* Final physical block of an accepted candidate: Reencode's AssignIndices +
 * optional refit + LogicalToPhysical, codec/dxt_image.cpp:900-905, :922-926. */
static uint64_t accepted_block(const block_ctx *b, const search_result *r) {
  if (!r->refit) return b->stb;
  uint8_t ep1[3], ep2[3];
  int valid;
  mo_refit(b->px, r->interp, ep1, ep2, &valid);
  return (uint64_t)pack565(ep1) | ((uint64_t)pack565(ep2) << 16) | ((uint64_t)r->interp << 32);
}

typedef struct {
  const uint8_t *rgb;
  int width, bw, bh, sa;
  int32_t thr;
  const uint64_t *stb, *prev;
  search_result *inter_res;
  int row0, row1;
  int64_t visited, refits;
} inter_job;

static void block_init(block_ctx *b, const uint8_t *rgb, int width, int bx, int by, uint64_t stb) {
  gather_block(rgb, width, bx, by, b->px);
  b->stb = stb;
  b->orig_err = mo_block_error(b->px, stb);
}

static void *inter_rows(void *arg) {
  inter_job *job = (inter_job *)arg;
  for (int by = job->row0; by < job->row1; ++by) {
    for (int bx = 0; bx < job->bw; ++bx) {
      size_t idx = (size_t)by * job->bw + bx;
      block_ctx b;
      block_init(&b, job->rgb, job->width, bx, by, job->stb[idx]);
      job->inter_res[idx] = inter_search(&b, bx, by, job->bw, job->bh, job->sa, job->prev,
                                         &job->visited, &job->refits);
    }
  }
  return NULL;
}

int mo_reencode_frame_mt(const uint8_t *rgb, int width, int height, const uint64_t *stb_blocks,
                         const uint64_t *prev_final, int search_area, int32_t err_threshold,
                         uint64_t *final_blocks, uint8_t *motion, uint32_t *unique_palette,
                         uint32_t *n_unique, mo_stats *stats, int threads) {
  if (!rgb || !stb_blocks || !final_blocks || !motion || !unique_palette || !n_unique) return -1;
  if (width <= 0 || height <= 0 || (width & 3) || (height & 3)) return -1;
  if (search_area < 1 || search_area > 64) return -1;
  const int bw = width >> 2, bh = height >> 2;
  const size_t nblk = (size_t)bw * bh;
  mo_stats st;
  memset(&st, 0, sizeof(st));

  /* Inter results for every block first: the inter search reads only the
   * previous frame (codec/dxt_image.cpp:739), so its order does not matter. */
  search_result *inter_res = NULL;
  if (prev_final) {
    inter_res = (search_result *)malloc(nblk * sizeof(search_result));
    if (!inter_res) return -2;
    if (threads < 1) threads = 1;
    if (threads > bh) threads = bh;
    inter_job jobs[256];
    pthread_t tid[256];
    if (threads > 256) threads = 256;
    for (int t = 0; t < threads; ++t) {
      inter_job j = {rgb, width, bw, bh, search_area, err_threshold, stb_blocks, prev_final,
                     inter_res, bh * t / threads, bh * (t + 1) / threads, 0, 0};
      jobs[t] = j;
    }
    for (int t = 1; t < threads; ++t) pthread_create(&tid[t], NULL, inter_rows, &jobs[t]);
    inter_rows(&jobs[0]);
    for (int t = 1; t < threads; ++t) pthread_join(tid[t], NULL);
    for (int t = 0; t < threads; ++t) {
      st.inter_visited += jobs[t].visited;
      st.refits += jobs[t].refits;
    }
  }

  /* Raster loop of DXTImage::Reencode, codec/dxt_image.cpp:878-956. The
   * current frame's blocks start as the stb blocks and are overwritten as soon
   * as each block is accepted, which the intra search of later blocks reads. */
  memcpy(final_blocks, stb_blocks, nblk * sizeof(uint64_t));
  uint32_t nu = 0;
  for (int by = 0; by < bh; ++by) {
    for (int bx = 0; bx < bw; ++bx) {
      size_t idx = (size_t)by * bw + bx;
      block_ctx b;
      block_init(&b, rgb, width, bx, by, stb_blocks[idx]);
      if (prev_final) {
        search_result r = inter_res[idx];
        if (r.min_err <= err_threshold) {
          final_blocks[idx] = accepted_block(&b, &r);
          motion[2 * idx + 0] = (uint8_t)(r.mx | 0x80);
          motion[2 * idx + 1] = (uint8_t)(r.my | 0x80);
          st.n_inter++;
          continue;
        }
      }
      search_result r = intra_search(&b, bx, by, bw, bh, search_area, final_blocks,
                                     &st.intra_visited, &st.refits);
      if (r.min_err <= err_threshold) {
        final_blocks[idx] = accepted_block(&b, &r);
        motion[2 * idx + 0] = (uint8_t)r.mx;
        motion[2 * idx + 1] = (uint8_t)r.my;
        st.n_intra++;
        continue;
      }
      motion[2 * idx + 0] = 255;
      motion[2 * idx + 1] = 255;
      unique_palette[nu++] = (uint32_t)(stb_blocks[idx] >> 32);
      st.n_unique++;
    }
  }
  *n_unique = nu;
  free(inter_res);
  if (stats) *stats = st;
  return 0;
}

int mo_reencode_frame(const uint8_t *rgb, int width, int height, const uint64_t *stb_blocks,
                      const uint64_t *prev_final, int search_area, int32_t err_threshold,
                      uint64_t *final_blocks, uint8_t *motion, uint32_t *unique_palette,
                      uint32_t *n_unique, mo_stats *stats) {
  return mo_reencode_frame_mt(rgb, width, height, stb_blocks, prev_final, search_area,
                              err_threshold, final_blocks, motion, unique_palette, n_unique, stats,
                              1);
}

/* DXTImage::PSNR, codec/dxt_image.cpp:363-383, over the final logical blocks:
 * a refit block keeps its 8-bit (snapped) endpoints, every other block is
 * PhysicalToLogical of its stb block. A block differs from its stb block
 * exactly when it was accepted with a refit. */
double mo_frame_psnr(const uint8_t *rgb, int width, int height, const uint64_t *final_blocks,
                     const uint64_t *stb_blocks) {
  const int bw = width >> 2, bh = height >> 2;
  double mse = 0.0;
  uint8_t *pal = (uint8_t *)malloc((size_t)bw * bh * 12);
  if (!pal) return -1.0;
  for (int by = 0; by < bh; ++by) {
    for (int bx = 0; bx < bw; ++bx) {
      size_t idx = (size_t)by * bw + bx;
      uint8_t p[4][3];
      if (final_blocks[idx] != stb_blocks[idx]) {
        uint8_t px[48], e1[3], e2[3];
        int valid;
        gather_block(rgb, width, bx, by, px);
        refit_endpoints(px, (uint32_t)(final_blocks[idx] >> 32), e1, e2);
        refit_palette(e1, e2, p);
        (void)valid;
      } else {
        block_palette(final_blocks[idx], p);
      }
      memcpy(pal + idx * 12, p, 12);
    }
  }
  for (int y = 0; y < height; y++) {
    for (int x = 0; x < width; x++) {
      size_t idx = (size_t)(y / 4) * bw + (x / 4);
      int k = (int)((final_blocks[idx] >> (32 + 2 * ((y % 4) * 4 + (x % 4)))) & 3);
      for (int c = 0; c < 3; c++) {
        double d = (double)rgb[((size_t)y * width + x) * 3 + c] - (double)pal[idx * 12 + k * 3 + c];
        mse += d * d;
      }
    }
  }
  free(pal);
  mse /= (double)(width * height);
  return 10.0 * log10((3.0 * 255.0 * 255.0) / mse);
}

/* Squared error of a frame against what a DXT1 decoder shows for its physical
 * blocks: every block's palette is PhysicalToLogical's (codec/dxt_image.cpp:198-227:
 * Decode565 of both endpoints, LerpChannels 1/3 and 2/3 when ep1 > ep2, else
 * the midpoint and black), whatever 8-bit endpoints a refit kept in the
 * encoder's logical blocks. This is the quantity DXTImage::PSNR
 * (:363-383) measures when every logical block is PhysicalToLogical of its
 * physical block, as after the constructor (:419-434). */
uint64_t mo_decoded_sse(const uint8_t *rgb, int width, int height, const uint64_t *blocks) {
  const int bw = width >> 2, bh = height >> 2;
  uint64_t sse = 0;
  for (int by = 0; by < bh; ++by) {
    for (int bx = 0; bx < bw; ++bx) {
      const uint64_t b = blocks[(size_t)by * bw + bx];
      uint8_t pal[4][3], px[48];
      block_palette(b, pal);
      gather_block(rgb, width, bx, by, px);
      for (int i = 0; i < 16; ++i) {
        const int k = (int)((b >> (32 + 2 * i)) & 3);
        for (int c = 0; c < 3; ++c) {
          const int d = (int)px[3 * i + c] - (int)pal[k][c];
          sse += (uint64_t)(d * d);
        }
      }
    }
  }
  return sse;
}
