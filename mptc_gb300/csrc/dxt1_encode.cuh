// K-a: stb_dxt DXT1 encode (alpha=0, STB_DXT_HIGHQUAL) of every 4x4 block of
// an RGB8 frame, bit-identical to Include/stb_dxt.h v1.04 as compiled on
// x86-64 (SSE float, no fused multiply-add).
//
// One thread per block. Every float/double step of the reference is written
// with an explicit round-to-nearest intrinsic so that nvcc can never contract a
// multiply and an add into an FMA (the file is also built with -fmad=false).
#pragma once
#include <cstdint>

namespace mptc {

// stb__OMatch5 / stb__OMatch6 (Include/stb_dxt.h:59-60, built by
// stb__PrepareOptTable :111-137); filled from the host at context creation.
__constant__ uint8_t c_omatch5[256][2];
__constant__ uint8_t c_omatch6[256][2];

// stb__Mul8Bit, Include/stb_dxt.h:64-68
__device__ __forceinline__ int stb_mul8bit(int a, int b) {
  int t = a * b + 128;
  return (t + (t >> 8)) >> 8;
}

// stb__As16Bit, Include/stb_dxt.h:82-85
__device__ __forceinline__ uint32_t stb_as16bit(int r, int g, int b) {
  return (uint32_t)((stb_mul8bit(r, 31) << 11) + (stb_mul8bit(g, 63) << 5) + stb_mul8bit(b, 31));
}

// stb__From16Bit with the Expand5/Expand6 tables written out, :70-80, :596-600
__device__ __forceinline__ void stb_from16(uint32_t v, int c[3]) {
  int r = (int)((v >> 11) & 31), g = (int)((v >> 5) & 63), b = (int)(v & 31);
  c[0] = (r << 3) | (r >> 2);
  c[1] = (g << 2) | (g >> 4);
  c[2] = (b << 3) | (b >> 2);
}

__device__ __forceinline__ int px_r(uint32_t p) { return (int)(p & 0xFF); }
__device__ __forceinline__ int px_g(uint32_t p) { return (int)((p >> 8) & 0xFF); }
__device__ __forceinline__ int px_b(uint32_t p) { return (int)((p >> 16) & 0xFF); }

// stb__MatchColorsBlock, no-dither branch, Include/stb_dxt.h:176-215
__device__ uint32_t stb_match_colors(const uint32_t px[16], uint32_t max16, uint32_t min16) {
  int c0[3], c1[3], c2[3], c3[3];
  stb_from16(max16, c0);
  stb_from16(min16, c1);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    c2[k] = (2 * c0[k] + c1[k]) / 3;  // stb__Lerp13 without rounding bias, :88-98
    c3[k] = (2 * c1[k] + c0[k]) / 3;
  }
  const int dr = c0[0] - c1[0], dg = c0[1] - c1[1], db = c0[2] - c1[2];
  const int s0 = c0[0] * dr + c0[1] * dg + c0[2] * db;
  const int s1 = c1[0] * dr + c1[1] * dg + c1[2] * db;
  const int s2 = c2[0] * dr + c2[1] * dg + c2[2] * db;
  const int s3 = c3[0] * dr + c3[1] * dg + c3[2] * db;
  const int c0p = (s1 + s3) >> 1, halfp = (s3 + s2) >> 1, c3p = (s2 + s0) >> 1;
  uint32_t mask = 0;
#pragma unroll
  for (int i = 15; i >= 0; --i) {
    const int dot = px_r(px[i]) * dr + px_g(px[i]) * dg + px_b(px[i]) * db;
    mask <<= 2;
    if (dot < halfp)
      mask |= (dot < c0p) ? 1u : 3u;
    else
      mask |= (dot < c3p) ? 2u : 0u;
  }
  return mask;
}

// stb__OptimizeColorsBlock, Include/stb_dxt.h:273-375
__device__ void stb_optimize_colors(const uint32_t px[16], uint32_t *pmax16, uint32_t *pmin16) {
  int mu[3], mn[3], mx[3];
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    const int sh = 8 * ch;
    int v0 = (int)((px[0] >> sh) & 0xFF);
    int muv = v0, minv = v0, maxv = v0;
#pragma unroll
    for (int i = 1; i < 16; ++i) {
      int v = (int)((px[i] >> sh) & 0xFF);
      muv += v;
      if (v < minv)
        minv = v;
      else if (v > maxv)
        maxv = v;
    }
    mu[ch] = (muv + 8) >> 4;
    mn[ch] = minv;
    mx[ch] = maxv;
  }
  int cov0 = 0, cov1 = 0, cov2 = 0, cov3 = 0, cov4 = 0, cov5 = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int r = px_r(px[i]) - mu[0], g = px_g(px[i]) - mu[1], b = px_b(px[i]) - mu[2];
    cov0 += r * r;
    cov1 += r * g;
    cov2 += r * b;
    cov3 += g * g;
    cov4 += g * b;
    cov5 += b * b;
  }
  // covf = cov / 255.0f, then four power iterations with left-to-right sums
  const float f0 = __fdiv_rn(__int2float_rn(cov0), 255.0f);
  const float f1 = __fdiv_rn(__int2float_rn(cov1), 255.0f);
  const float f2 = __fdiv_rn(__int2float_rn(cov2), 255.0f);
  const float f3 = __fdiv_rn(__int2float_rn(cov3), 255.0f);
  const float f4 = __fdiv_rn(__int2float_rn(cov4), 255.0f);
  const float f5 = __fdiv_rn(__int2float_rn(cov5), 255.0f);
  float vfr = __int2float_rn(mx[0] - mn[0]);
  float vfg = __int2float_rn(mx[1] - mn[1]);
  float vfb = __int2float_rn(mx[2] - mn[2]);
#pragma unroll
  for (int iter = 0; iter < 4; ++iter) {
    const float r = __fadd_rn(__fadd_rn(__fmul_rn(vfr, f0), __fmul_rn(vfg, f1)), __fmul_rn(vfb, f2));
    const float g = __fadd_rn(__fadd_rn(__fmul_rn(vfr, f1), __fmul_rn(vfg, f3)), __fmul_rn(vfb, f4));
    const float b = __fadd_rn(__fadd_rn(__fmul_rn(vfr, f2), __fmul_rn(vfg, f4)), __fmul_rn(vfb, f5));
    vfr = r;
    vfg = g;
    vfb = b;
  }
  // magn in double (fabs of the float values)
  double magn = fabs((double)vfr);
  if (fabs((double)vfg) > magn) magn = fabs((double)vfg);
  if (fabs((double)vfb) > magn) magn = fabs((double)vfb);
  int v_r, v_g, v_b;
  if (magn < 4.0) {
    v_r = 299;
    v_g = 587;
    v_b = 114;
  } else {
    magn = __ddiv_rn(512.0, magn);
    // |vf * magn| <= 512: the truncating conversion never leaves int range
    v_r = __double2int_rz(__dmul_rn((double)vfr, magn));
    v_g = __double2int_rz(__dmul_rn((double)vfg, magn));
    v_b = __double2int_rz(__dmul_rn((double)vfb, magn));
  }
  int mind = 0x7fffffff, maxd = -0x7fffffff, imin = 0, imax = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int dot = px_r(px[i]) * v_r + px_g(px[i]) * v_g + px_b(px[i]) * v_b;
    if (dot < mind) {
      mind = dot;
      imin = i;
    }
    if (dot > maxd) {
      maxd = dot;
      imax = i;
    }
  }
  uint32_t pmx = 0, pmnv = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {  // register-resident select instead of a dynamic index
    pmx = (i == imax) ? px[i] : pmx;
    pmnv = (i == imin) ? px[i] : pmnv;
  }
  *pmax16 = stb_as16bit(px_r(pmx), px_g(pmx), px_b(pmx));
  *pmin16 = stb_as16bit(px_r(pmnv), px_g(pmnv), px_b(pmnv));
}

// stb__sclamp, :377-383 (the argument always fits an int here)
__device__ __forceinline__ uint32_t stb_sclamp(float y, int hi) {
  int x = __float2int_rz(y);
  x = x < 0 ? 0 : x;
  return (uint32_t)(x > hi ? hi : x);
}

// stb__RefineBlock, Include/stb_dxt.h:388-464
__device__ bool stb_refine(const uint32_t px[16], uint32_t *pmax16, uint32_t *pmin16, uint32_t mask) {
  const uint32_t old_min = *pmin16, old_max = *pmax16;
  uint32_t min16, max16;
  if ((mask ^ (mask << 2)) < 4u) {
    int r = 8, g = 8, b = 8;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      r += px_r(px[i]);
      g += px_g(px[i]);
      b += px_b(px[i]);
    }
    r >>= 4;
    g >>= 4;
    b >>= 4;
    max16 = ((uint32_t)c_omatch5[r][0] << 11) | ((uint32_t)c_omatch6[g][0] << 5) | c_omatch5[b][0];
    min16 = ((uint32_t)c_omatch5[r][1] << 11) | ((uint32_t)c_omatch6[g][1] << 5) | c_omatch5[b][1];
  } else {
    // w1Tab {3,0,2,1}; prods {0x090000,0x000900,0x040102,0x010402}
    int akku = 0, a1r = 0, a1g = 0, a1b = 0, a2r = 0, a2g = 0, a2b = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const uint32_t step = (mask >> (2 * i)) & 3u;
      const int w1 = step == 0 ? 3 : step == 1 ? 0 : step == 2 ? 2 : 1;
      const int prod = step == 0 ? 0x090000 : step == 1 ? 0x000900 : step == 2 ? 0x040102 : 0x010402;
      const int r = px_r(px[i]), g = px_g(px[i]), b = px_b(px[i]);
      akku += prod;
      a1r += w1 * r;
      a1g += w1 * g;
      a1b += w1 * b;
      a2r += r;
      a2g += g;
      a2b += b;
    }
    a2r = 3 * a2r - a1r;
    a2g = 3 * a2g - a1g;
    a2b = 3 * a2b - a1b;
    const int xx = akku >> 16, yy = (akku >> 8) & 0xff, xy = akku & 0xff;
    // frb = 3.0f * 31.0f / 255.0f / (xx*yy - xy*xy); fg = frb * 63.0f / 31.0f
    const float frb = __fdiv_rn(__fdiv_rn(93.0f, 255.0f), __int2float_rn(xx * yy - xy * xy));
    const float fg = __fdiv_rn(__fmul_rn(frb, 63.0f), 31.0f);
    max16 = stb_sclamp(__fadd_rn(__fmul_rn(__int2float_rn(a1r * yy - a2r * xy), frb), 0.5f), 31) << 11;
    max16 |= stb_sclamp(__fadd_rn(__fmul_rn(__int2float_rn(a1g * yy - a2g * xy), fg), 0.5f), 63) << 5;
    max16 |= stb_sclamp(__fadd_rn(__fmul_rn(__int2float_rn(a1b * yy - a2b * xy), frb), 0.5f), 31);
    min16 = stb_sclamp(__fadd_rn(__fmul_rn(__int2float_rn(a2r * xx - a1r * xy), frb), 0.5f), 31) << 11;
    min16 |= stb_sclamp(__fadd_rn(__fmul_rn(__int2float_rn(a2g * xx - a1g * xy), fg), 0.5f), 63) << 5;
    min16 |= stb_sclamp(__fadd_rn(__fmul_rn(__int2float_rn(a2b * xx - a1b * xy), frb), 0.5f), 31);
  }
  *pmin16 = min16;
  *pmax16 = max16;
  return old_min != min16 || old_max != max16;
}

// stb__CompressColorBlock with mode = STB_DXT_HIGHQUAL, Include/stb_dxt.h:467-538.
// px[i] = r | g<<8 | b<<16 | 0xFF<<24 (alpha forced to 0xFF as CompressRGB does).
__device__ uint64_t stb_encode_block(const uint32_t px[16]) {
  uint32_t mask, max16, min16;
  bool constant = true;
#pragma unroll
  for (int i = 1; i < 16; ++i) constant = constant && (px[i] == px[0]);
  if (constant) {
    const int r = px_r(px[0]), g = px_g(px[0]), b = px_b(px[0]);
    mask = 0xaaaaaaaau;
    max16 = ((uint32_t)c_omatch5[r][0] << 11) | ((uint32_t)c_omatch6[g][0] << 5) | c_omatch5[b][0];
    min16 = ((uint32_t)c_omatch5[r][1] << 11) | ((uint32_t)c_omatch6[g][1] << 5) | c_omatch5[b][1];
  } else {
    stb_optimize_colors(px, &max16, &min16);
    mask = (max16 != min16) ? stb_match_colors(px, max16, min16) : 0u;
    for (int it = 0; it < 2; ++it) {
      const uint32_t lastmask = mask;
      if (stb_refine(px, &max16, &min16, mask)) {
        if (max16 != min16) {
          mask = stb_match_colors(px, max16, min16);
        } else {
          mask = 0;
          break;
        }
      }
      if (mask == lastmask) break;
    }
  }
  if (max16 < min16) {
    const uint32_t t = min16;
    min16 = max16;
    max16 = t;
    mask ^= 0x55555555u;
  }
  return (uint64_t)max16 | ((uint64_t)min16 << 16) | ((uint64_t)mask << 32);
}

// CompressedBlock::Error of a physical block (codec/dxt_image.cpp:258-276) on
// its PhysicalToLogical palette (:198-227): 4-colour when ep1 > ep2, else
// 3-colour with colour 3 black.
__device__ int block_error_physical(const uint32_t px[16], uint64_t blk) {
  const uint32_t e1 = (uint32_t)(blk & 0xFFFF), e2 = (uint32_t)((blk >> 16) & 0xFFFF);
  const uint32_t idx = (uint32_t)(blk >> 32);
  int a[3], b[3], p2[3], p3[3];
  stb_from16(e1, a);
  stb_from16(e2, b);
  const bool four = e1 > e2;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    p2[c] = four ? (2 * a[c] + b[c]) / 3 : (a[c] + b[c]) / 2;
    p3[c] = four ? (a[c] + 2 * b[c]) / 3 : 0;
  }
  uint32_t err = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint32_t k = (idx >> (2 * i)) & 3u;
    const int pr = k == 0 ? a[0] : k == 1 ? b[0] : k == 2 ? p2[0] : p3[0];
    const int pg = k == 0 ? a[1] : k == 1 ? b[1] : k == 2 ? p2[1] : p3[1];
    const int pb = k == 0 ? a[2] : k == 1 ? b[2] : k == 2 ? p2[2] : p3[2];
    const int dr = px_r(px[i]) - pr, dg = px_g(px[i]) - pg, db = px_b(px[i]) - pb;
    err += (uint32_t)(dr * dr + dg * dg + db * db);
  }
  return (int)(err / 48u);
}

// Gathers block (bx, by) of an RGB8 frame (row pitch = width*3 bytes, a
// multiple of 4) into 16 packed pixels. Rows are read as three aligned words.
__device__ __forceinline__ void load_block_px(const uint8_t *__restrict__ rgb, int width, int bx,
                                              int by, uint32_t px[16]) {
  const size_t pitch = (size_t)width * 3;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint32_t *row = reinterpret_cast<const uint32_t *>(rgb + (size_t)(4 * by + r) * pitch + 12 * (size_t)bx);
    const uint32_t w0 = __ldg(row + 0), w1 = __ldg(row + 1), w2 = __ldg(row + 2);
    // bytes: r0 g0 b0 r1 | g1 b1 r2 g2 | b2 r3 g3 b3
    px[4 * r + 0] = (w0 & 0x00FFFFFFu) | 0xFF000000u;
    px[4 * r + 1] = (w0 >> 24) | ((w1 & 0xFFFFu) << 8) | 0xFF000000u;
    px[4 * r + 2] = (w1 >> 16) | ((w2 & 0xFFu) << 16) | 0xFF000000u;
    px[4 * r + 3] = (w2 >> 8) | 0xFF000000u;
  }
}

// One thread per block: stb block and its reference error.
__global__ void __launch_bounds__(128) dxt1_encode_kernel(const uint8_t *__restrict__ rgb, int width,
                                                          int bw, int nblk, uint64_t *__restrict__ blocks,
                                                          int32_t *__restrict__ orig_err) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nblk; idx += gridDim.x * blockDim.x) {
    const int by = idx / bw, bx = idx - by * bw;
    uint32_t px[16];
    load_block_px(rgb, width, bx, by, px);
    const uint64_t blk = stb_encode_block(px);
    blocks[idx] = blk;
    if (orig_err) orig_err[idx] = block_error_physical(px, blk);
  }
}

}  // namespace mptc
