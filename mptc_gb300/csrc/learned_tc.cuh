// Learned candidate proposal, the search half: window scoring on the
// fifth-generation tensor cores (tcgen05) — block embeddings against the
// embeddings of the distinct index words around each tile of blocks (the
// tile's word palette), each block's top-K distinct window words taken by
// warp reductions — then the exact test of the K proposals with the reference's
// selection rule, and the exhaustive search of the blocks none passed.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>

#include "learned_common.cuh"
#include "search.cuh"
#include "tc_sm100.cuh"

namespace mptc {

// ---- window scoring + top-K ------------------------------------------------------
// Tiles of 16 block rows x 8 block columns; M row m = 16c + r holds the
// block at column c, row r of the tile (one TMEM lane each). The union of the
// tile's inter windows spans UR = 16 + 2sa - 1 <= 31 rows and UC = 8 + 2sa - 1
// <= 23 columns of the previous frame (sa <= 8). Final blocks reuse
// dictionary words, so a union holds few distinct index words (45-110 on
// 1080p content, against 713 positions) and a window about 33-55.
//
// Per tile, in shared memory:
//  1. the palette: the union's distinct words by an open-addressed hash
//     table (1024 slots, linear probing), numbered in slot order, each with
//     the G row of its word (read with the words, a tile ahead); every union
//     position's palette id;
//  2. per slice of SL palette entries (the dictionary slice of a stage;
//     SL = 16 ROWS): the slice's G rows gathered in the 128-byte-swizzled
//     K-major layout and one tcgen05 MMA of the tile's F rows (eight TMA
//     copies of one block column each) against them into TMEM. Meanwhile the
//     four threads of each block (warps w, w + 4, w + 8, w + 12 share TMEM lane
//     quadrant w) scan four window rows each, last position first, and leave
//     in byte g of word (block, entry) 1 + the entry's first offset in rows
//     4g .. 4g + 3 (scan order): the lowest nonzero byte gives the first scan position
//     (rows ascending, columns ascending, the reference's scan order) with
//     plain stores. A cell whose word is that of its left neighbour, or of
//     the cell above in the same four rows, is skipped: that neighbour comes
//     later and holds an earlier position;
//  3. each thread ranks 32 entries of its block straight from TMEM: a rank
//     key packs the score's order key (an integer that orders as the float
//     does) in its 24 leading bits with 255 - position below, so one unsigned
//     comparison orders by score and, among scores equal in those bits, by
//     first position; absent words rank 0. Sorting networks of max/min keep
//     the thread's best K, then one thread per block merges the four lists
//     (and, after the first slice, the block's best K so far). Palette
//     entries are distinct words: nothing to deduplicate.
constexpr int kScoreTileW = 8, kScoreTileH = 16;
constexpr int kScoreWarps = 16, kScoreThreads = 32 * kScoreWarps;
constexpr int kPalSlots = 1024;  // hash slots (> the 713 union positions at sa = 8)
// A union position's palette id (0x3FFF: outside the frame) with flags: the
// word is that of the position to the left, of the position above.
constexpr uint16_t kPidMask = 0x3FFFu, kSameLeft = 0x8000u, kSameAbove = 0x4000u;

struct ScoreArgs {
  int bw, bh, sa;
  const uint32_t *words;      // the previous frame's index words, words[pos * word_stride]
  int word_stride;
  const __nv_bfloat16 *gemb;  // G rows, [rows][64]
  const uint32_t *rows;       // G row of the word at each position (NULL: row = position)
  uint16_t *topk;             // n x kMaxK window positions, best first
  uint32_t *status;           // device status word
};

// A launch covers the frames of up to kMaxBatch jobs (the streams of a
// batch, or one): score tiles are numbered across the jobs and CTAs take them
// from one counter. Job j's F rows are reached through its tensor map (boxes
// of one block column, 16 rows).
struct ScoreBatch {
  int n;
  int tile_end[kMaxBatch];
  ScoreArgs a[kMaxBatch];
  CUtensorMap tmF[kMaxBatch];
  uint32_t *next;  // tile counter (zero before the launch)
};

// A score's order key: larger float, larger key; every float but the
// all-ones NaN pattern has a key > 0 (every finite score one >= 2^23).
__device__ __forceinline__ uint32_t score_key(uint32_t u) {
  return u ^ ((uint32_t)((int32_t)u >> 31) | 0x80000000u);
}

// The rank key of a present word: the order key's 24 leading bits, then
// 255 - position (larger ranks first: higher score, then earlier position).
__device__ __forceinline__ uint32_t rank_key(float score, uint32_t pos) {
  return (score_key(__float_as_uint(score)) & 0xFFFFFF00u) | (255u - pos);
}

__device__ __forceinline__ uint32_t pal_hash(uint32_t word) { return (word * 2654435761u) >> 22; }

__device__ __forceinline__ void cas_desc(uint32_t &a, uint32_t &b) {
  const uint32_t hi = max(a, b), lo = min(a, b);
  a = hi;
  b = lo;
}

// Bitonic sort of a[0, N), descending (N a power of two; registers).
template <int N>
__device__ __forceinline__ void sort_desc(uint32_t *a) {
#pragma unroll
  for (int k = 2; k <= N; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const int l = i ^ j;
        if (l > i) {
          if ((i & k) == 0)
            cas_desc(a[i], a[l]);
          else
            cas_desc(a[l], a[i]);
        }
      }
    }
  }
}

// a[0, K) := the K largest of a[0, K) and b[0, K), descending (both
// descending): the elementwise maximum against b reversed is a bitonic
// sequence holding them, which a bitonic merge sorts.
template <int K>
__device__ __forceinline__ void merge_top(uint32_t *a, const uint32_t *b) {
#pragma unroll
  for (int i = 0; i < K; ++i) a[i] = max(a[i], b[K - 1 - i]);
#pragma unroll
  for (int j = K >> 1; j > 0; j >>= 1) {
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int l = i ^ j;
      if (l > i) cas_desc(a[i], a[l]);
    }
  }
}

// Shared-memory layout of the scoring kernel (byte offsets from a 1024-byte
// aligned base) for slices of SL palette entries and K proposals.
template <int SL, int K>
struct ScoreSmem {
  static constexpr int kRow = SL + 4;  // words per block row of first-offset bytes
  static constexpr size_t F = 0;
  static constexpr size_t G = F + tc::kTileBytes;
  static constexpr size_t First = G + (size_t)SL * 128;
  // rank keys, block index fastest (a warp's 32 blocks in 32 banks):
  // Part [4 groups x K][128 blocks], Carry [K][128 blocks]
  static constexpr size_t Part = First + (size_t)128 * kRow * 4;
  static constexpr size_t Carry = Part + (size_t)128 * 4 * K * 4;
  static constexpr size_t Hash = Carry + (size_t)128 * K * 4;
  static constexpr size_t Slot = Hash + (size_t)kPalSlots * 8;      // union position -> slot -> palette id
  static constexpr size_t PalIdx = Slot + (size_t)kPalSlots * 2;    // slot -> palette id
  static constexpr size_t PalRow = PalIdx + (size_t)kPalSlots * 2;  // palette id -> G row
  static constexpr size_t Pid = PalRow + (size_t)kPalSlots * 4;      // union position -> palette id | flags
  static constexpr size_t WarpTot = Pid + (size_t)kPalSlots * 2;
  static constexpr size_t Bars = WarpTot + kScoreWarps * 4;
  static constexpr size_t Bytes = Bars + 64;
};

template <int ROWS, int K>
constexpr size_t score_smem_bytes() {
  return 1024 + ScoreSmem<16 * ROWS, K>::Bytes;
}

using tc::kTileBytes;

template <int ROWS, int K>
__global__ void __launch_bounds__(kScoreThreads, 1) score_topk_tc_kernel(const __grid_constant__ ScoreBatch batch) {
  constexpr int SL = 16 * ROWS;
  using L = ScoreSmem<SL, K>;
  constexpr int kRow = L::kRow;
  constexpr uint32_t kFColBytes = 16 * 128;  // one block column of the F tile
  extern __shared__ uint8_t dsm[];
  uint8_t *sm = tc::align_1024(dsm);
  uint8_t *const sF = sm + L::F;
  uint8_t *const sG = sm + L::G;
  uint32_t *const sFirst = reinterpret_cast<uint32_t *>(sm + L::First);
  uint32_t *const sPart = reinterpret_cast<uint32_t *>(sm + L::Part);
  uint32_t *const sCarry = reinterpret_cast<uint32_t *>(sm + L::Carry);
  unsigned long long *const sHash = reinterpret_cast<unsigned long long *>(sm + L::Hash);
  uint16_t *const sSlot = reinterpret_cast<uint16_t *>(sm + L::Slot);
  uint16_t *const sPalIdx = reinterpret_cast<uint16_t *>(sm + L::PalIdx);
  uint32_t *const sPalRow = reinterpret_cast<uint32_t *>(sm + L::PalRow);
  uint16_t *const sPid = reinterpret_cast<uint16_t *>(sm + L::Pid);
  uint32_t *const sWarpTot = reinterpret_cast<uint32_t *>(sm + L::WarpTot);
  uint64_t *const bar = reinterpret_cast<uint64_t *>(sm + L::Bars);  // F, M
  uint32_t *const tslot = reinterpret_cast<uint32_t *>(bar + 2);
  volatile uint32_t *abort_flag = tslot + 1;
  volatile int *s_tile = reinterpret_cast<volatile int *>(tslot + 2);
  volatile int *s_next = reinterpret_cast<volatile int *>(tslot + 3);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_init(bar + 1, 1);
    *abort_flag = 0;
    tc::mbar_fence_init();
  }
  for (int i = tid; i < 128 * kRow / 4; i += kScoreThreads)
    reinterpret_cast<uint4 *>(sFirst)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (warp == 0) tc::tmem_alloc(tslot, SL < 32 ? 32 : SL);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc::idesc_bf16(128, SL);
  // this thread's block (TMEM lane), its window rows 4g .. 4g + 3 and entries
  // 32g .. 32g + 31 of a slice
  const int quad = warp & 3, g = warp >> 2;
  const int mt = 32 * quad + lane, ct = mt >> 4, rt = mt & 15;
  uint32_t *const myfirst = sFirst + mt * kRow;
  // phase parities: bit 0 F, bit 1 the MMA
  uint32_t phase = 0;
  auto wait = [&](uint64_t *b, int bit) {
    if (!tc::mbar_wait(b, (phase >> bit) & 1u, abort_flag)) *abort_flag = 1;
    phase ^= 1u << bit;
  };
  struct TileAt {
    int jb, tx0, ty0;
  };
  auto locate = [&](int gt) {
    int jb = 0;
    while (gt >= batch.tile_end[jb]) ++jb;
    const ScoreArgs &a = batch.a[jb];
    const int tile = gt - (jb ? batch.tile_end[jb - 1] : 0);
    const int tiles_x = (a.bw + kScoreTileW - 1) / kScoreTileW;
    return TileAt{jb, (tile % tiles_x) * kScoreTileW, (tile / tiles_x) * kScoreTileH};
  };
  auto load_f = [&](int gt) {  // thread 0: the tile's F rows, one block column per copy
    const TileAt t = locate(gt);
    tc::mbar_arrive_expect_tx(bar, kTileBytes);
#pragma unroll 1
    for (int cc = 0; cc < kScoreTileW; ++cc)
      tc::tma_load_3d(sF + cc * kFColBytes, &batch.tmF[t.jb], 0, t.tx0 + cc, t.ty0, bar);
  };
  const int total = batch.tile_end[batch.n - 1];
  // the union words of a tile and their G rows, read ahead: thread tid
  // holds cells tid and tid + 512 (713 at most) of tile pf
  constexpr int kCellsPerThread = (kPalSlots + kScoreThreads - 1) / kScoreThreads;
  uint32_t pw[kCellsPerThread], prow[kCellsPerThread];
  int pf = -1;
  auto read_words = [&](int gt) {
    const TileAt t = locate(gt);
    const ScoreArgs &a = batch.a[t.jb];
    const int UC = kScoreTileW + 2 * a.sa - 1, nU = (kScoreTileH + 2 * a.sa - 1) * UC;
#pragma unroll
    for (int i = 0; i < kCellsPerThread; ++i) {
      const int q = tid + i * kScoreThreads;
      pw[i] = 0;
      prow[i] = 0;
      if (q < nU) {
        const int uy = q / UC, ux = q - uy * UC;
        const int gy = t.ty0 - a.sa + uy, gx = t.tx0 - a.sa + ux;
        if (gy >= 0 && gy < a.bh && gx >= 0 && gx < a.bw) {
          const uint32_t pos = (uint32_t)gy * (uint32_t)a.bw + (uint32_t)gx;
          pw[i] = __ldg(a.words + (size_t)pos * a.word_stride);
          prow[i] = a.rows ? __ldg(a.rows + pos) : pos;
        }
      }
    }
    pf = gt;
  };
  for (int i = tid; i < kPalSlots; i += kScoreThreads) sHash[i] = 0ull;
  if (tid == 0) {
    const int gt = (int)atomicAdd(batch.next, 1u);
    *s_tile = gt;
    if (gt < total) load_f(gt);
  }
  for (;;) {
    // one decision for the whole CTA: no thread sets the abort flag between
    // this barrier's reads
    const bool stop = __syncthreads_or(*abort_flag != 0) != 0;
    const int gt = *s_tile;
    if (gt >= total || stop) break;
    if (tid == 0) *s_next = (int)atomicAdd(batch.next, 1u);  // the next tile, claimed now
    const TileAt t = locate(gt);
    const ScoreArgs &a = batch.a[t.jb];
    const int tx0 = t.tx0, ty0 = t.ty0, sa = a.sa, w2 = 2 * sa;
    const int UC = kScoreTileW + w2 - 1, nU = (kScoreTileH + w2 - 1) * UC;
    if (pf != gt) read_words(gt);
    // 1. the palette (the table was cleared after the previous tile's numbering)
#pragma unroll
    for (int i = 0; i < kCellsPerThread; ++i) {
      const int q = tid + i * kScoreThreads;
      if (q >= nU) break;
      const int uy = q / UC, ux = q - uy * UC;
      const int gy = ty0 - sa + uy, gx = tx0 - sa + ux;
      uint16_t slot = 0xFFFFu;
      if (gy >= 0 && gy < a.bh && gx >= 0 && gx < a.bw) {
        const uint32_t word = pw[i];
        const unsigned long long entry = ((unsigned long long)word << 32) | (unsigned long long)(prow[i] + 1u);
        uint32_t h = pal_hash(word);
        for (int it = 0; it < kPalSlots; ++it) {  // the table never fills: it ends
          const unsigned long long old = atomicCAS(sHash + h, 0ull, entry);
          if (old == 0ull || (uint32_t)(old >> 32) == word) break;
          h = (h + 1) & (kPalSlots - 1);
        }
        slot = (uint16_t)h;
      }
      sSlot[q] = slot;
    }
    __syncthreads();
    // the next tile's words, in flight while this tile is scored
    const int nt = *s_next;
    if (nt < total) read_words(nt);
    int npal;
    {
      const int s0 = 64 * warp + lane, s1 = s0 + 32;
      const unsigned long long h0 = sHash[s0], h1 = sHash[s1];
      const uint32_t b0 = __ballot_sync(kFull, h0 != 0ull), b1 = __ballot_sync(kFull, h1 != 0ull);
      const uint32_t lt = (1u << lane) - 1u;
      if (lane == 0) sWarpTot[warp] = __popc(b0) + __popc(b1);
      __syncthreads();
      int base = 0;
      npal = 0;
#pragma unroll
      for (int w = 0; w < kScoreWarps; ++w) {
        const int tw = (int)sWarpTot[w];
        base += w < warp ? tw : 0;
        npal += tw;
      }
      if (h0) {
        const int id = base + __popc(b0 & lt);
        sPalIdx[s0] = (uint16_t)id;
        sPalRow[id] = (uint32_t)h0 - 1u;
      }
      if (h1) {
        const int id = base + __popc(b0) + __popc(b1 & lt);
        sPalIdx[s1] = (uint16_t)id;
        sPalRow[id] = (uint32_t)h1 - 1u;
      }
    }
    __syncthreads();
    // slice 0's G rows in flight during the palette ids pass
    constexpr int kGPerThread = SL * 8 / kScoreThreads;
    uint4 gv[kGPerThread];
    const int nc0 = min(SL, npal);
#pragma unroll
    for (int i = 0; i < kGPerThread; ++i) {
      const int c = tid + i * kScoreThreads, e = c >> 3, j = c & 7;
      gv[i] = make_uint4(0u, 0u, 0u, 0u);
      if (e < nc0) gv[i] = __ldg(reinterpret_cast<const uint4 *>(a.gemb + (size_t)sPalRow[e] * kEmb) + j);
    }
    for (int q = tid; q < nU; q += kScoreThreads) {
      const uint16_t sl = sSlot[q];
      uint16_t v = kPidMask;
      if (sl != 0xFFFFu) {
        v = sPalIdx[sl];
        const int ux = q % UC;
        if (ux > 0 && sSlot[q - 1] == sl) v |= kSameLeft;
        if (q >= UC && sSlot[q - UC] == sl) v |= kSameAbove;
      }
      sPid[q] = v;
    }
    for (int i = tid; i < kPalSlots; i += kScoreThreads) sHash[i] = 0ull;  // for the next tile
#pragma unroll
    for (int i = 0; i < kGPerThread; ++i) {
      const int c = tid + i * kScoreThreads;
      *reinterpret_cast<uint4 *>(sG + tc::sw128_offset((uint32_t)(c >> 3), (uint32_t)(c & 7))) = gv[i];
    }
    tc::fence_async_smem();
    // 2.-3. slice by slice
    const int nsl = npal > 0 ? (npal + SL - 1) / SL : 1;
    const int bx = tx0 + ct, by = ty0 + rt;
    const bool t_in = bx < a.bw && by < a.bh;
#pragma unroll 1
    for (int sl = 0; sl < nsl; ++sl) {
      const int e0 = sl * SL, nc = min(SL, npal - e0);
      __syncthreads();  // palette ids and slice 0's G rows written; the previous slice's merge done
      if (sl > 0) {
        for (int i = tid; i < SL * 8; i += kScoreThreads) {
          const int e = i >> 3, j = i & 7;
          uint4 v = make_uint4(0u, 0u, 0u, 0u);
          if (e < nc) v = __ldg(reinterpret_cast<const uint4 *>(a.gemb + (size_t)sPalRow[e0 + e] * kEmb) + j);
          *reinterpret_cast<uint4 *>(sG + tc::sw128_offset((uint32_t)e, (uint32_t)j)) = v;
        }
        tc::fence_async_smem();
        __syncthreads();
      }
      if (tid == 0) {
        if (sl == 0) wait(bar, 0);
        tc::tc_fence_after();
        const uint32_t fa = tc::smem_addr(sF), ga = tc::smem_addr(sG);
#pragma unroll
        for (int k = 0; k < 4; ++k)
          tc::mma_bf16(tmem, tc::desc_sw128(fa + 32 * k), tc::desc_sw128(ga + 32 * k), idesc, k > 0);
        tc::mma_commit(bar + 1);
      }
      // first offsets of the slice entries in window rows 4g .. 4g + 3, the
      // last position first so the first one stays; a row's palette ids are
      // read before its stores
      if (t_in && 4 * g < w2) {
        uint8_t *const fb = reinterpret_cast<uint8_t *>(myfirst) + g;
#pragma unroll 1
        for (int wrow = min(4 * g + 3, w2 - 1); wrow >= 4 * g; --wrow) {
          const uint16_t *srow = sPid + (rt + wrow) * UC + ct;
          uint16_t v[16];
#pragma unroll
          for (int c = 0; c < 16; ++c) v[c] = c < w2 ? srow[c] : kPidMask;
          const uint32_t rb = (uint32_t)(wrow - 4 * g) * (uint32_t)w2 + 1u;
          const uint16_t up = wrow > 4 * g ? kSameAbove : (uint16_t)0;
#pragma unroll
          for (int c = 15; c >= 0; --c) {
            // absent (0x3FFF) or another slice: >= nc
            const uint32_t e = (uint32_t)(v[c] & kPidMask) - (uint32_t)e0;
            const bool later = (v[c] & (c > 0 ? (uint16_t)(kSameLeft | up) : up)) != 0;
            if (e < (uint32_t)nc && !later) fb[4 * e] = (uint8_t)(rb + (uint32_t)c);
          }
        }
      }
      wait(bar + 1, 1);
      tc::tc_fence_after();
      __syncthreads();  // first offsets complete
      // this thread's best K of its 32 entries
      if (32 * g < nc) {
        float v[32];
        tc::tmem_ld32(tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(32 * g), v);
        uint32_t rk[32];
        uint32_t *const fw = myfirst + 32 * g;
#pragma unroll
        for (int i = 0; i < 32; i += 4) {
          const uint4 f4 = *reinterpret_cast<const uint4 *>(fw + i);
          *reinterpret_cast<uint4 *>(fw + i) = make_uint4(0u, 0u, 0u, 0u);
          const uint32_t fv[4] = {f4.x, f4.y, f4.z, f4.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const uint32_t f = fv[u];
            const uint32_t sh = (uint32_t)max(__ffs((int)f) - 1, 0) & ~7u;  // lowest nonzero byte: the first group
            const uint32_t pos = (sh >> 3) * 4u * (uint32_t)w2 + ((f >> sh) & 0xFFu) - 1u;
            rk[i + u] = f ? rank_key(v[i + u], pos) : 0u;
          }
        }
#pragma unroll
        for (int c = 0; c < 32; c += K) sort_desc<K>(rk + c);
#pragma unroll
        for (int c = K; c < 32; c += K) merge_top<K>(rk, rk + c);
#pragma unroll
        for (int i = 0; i < K; ++i) sPart[(g * K + i) * 128 + mt] = rk[i];
      }
      tc::tc_fence_before();
      __syncthreads();  // partial lists written; TMEM and the F rows free
      const bool last = sl == nsl - 1;
      if (last && tid == 0) {  // the next tile's F rows
        *s_tile = nt;
        if (nt < total && !*abort_flag) load_f(nt);
      }
      if (g == 0 && t_in) {  // the block's best K: its four lists and the best K so far
        uint32_t best[K], other[K];
#pragma unroll
        for (int i = 0; i < K; ++i) best[i] = sPart[i * 128 + mt];
#pragma unroll
        for (int gg = 1; gg < 4; ++gg) {
          if (32 * gg < nc) {
#pragma unroll
            for (int i = 0; i < K; ++i) other[i] = sPart[(gg * K + i) * 128 + mt];
            merge_top<K>(best, other);
          }
        }
        if (sl > 0) {
#pragma unroll
          for (int i = 0; i < K; ++i) other[i] = sCarry[i * 128 + mt];
          merge_top<K>(best, other);
        }
        if (!last) {
#pragma unroll
          for (int i = 0; i < K; ++i) sCarry[i * 128 + mt] = best[i];
        } else {
          uint32_t o[kMaxK / 2];
#pragma unroll
          for (int i = 0; i < kMaxK; i += 2) {
            const uint32_t p0 = (i < K && best[i < K ? i : 0]) ? 255u - (best[i < K ? i : 0] & 0xFFu) : kNoProposal;
            const uint32_t p1 =
                (i + 1 < K && best[i + 1 < K ? i + 1 : 0]) ? 255u - (best[i + 1 < K ? i + 1 : 0] & 0xFFu) : kNoProposal;
            o[i / 2] = p0 | (p1 << 16);
          }
          uint4 *dst = reinterpret_cast<uint4 *>(a.topk + ((size_t)by * a.bw + bx) * kMaxK);
          dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
          dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_free(tmem, SL < 32 ? 32 : SL);
  if (tid == 0 && *abort_flag)
    for (int j = 0; j < batch.n; ++j) atomicOr(batch.a[j].status, kDevTimeout);
}

// ---- exact test of the proposals -------------------------------------------------
// A warp tests the K proposals of 32/K blocks at once (lane = block slot x
// proposal). Each proposal is evaluated exactly (refit, snap, validity, error;
// codec/dxt_image.cpp:258-349) and the reference's selection rule
// (codec/dxt_image.cpp:715-774: the first err_diff <= 0 in scan order ends its
// row, a later row's first err_diff < 0 replaces it, otherwise the first
// minimum) runs over the K proposal positions in closed form. A block whose
// selection passes the threshold becomes final with the reference's inter
// motion code; the others are listed for the exhaustive search.
// The frames of up to kMaxBatch jobs per launch: job j owns the block groups
// [group_end[j-1], group_end[j]) (a group: the 32/K blocks of one warp pass).
struct EvalBatch {
  int n;
  int group_end[kMaxBatch];
  SearchParams P[kMaxBatch];
  const uint16_t *topk[kMaxBatch];
  uint32_t *fb_count[kMaxBatch];  // zeroed fallback counter
  uint32_t *fb_list[kMaxBatch];   // room for every block of the frame
};

template <int K, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) learned_eval_kernel(const __grid_constant__ EvalBatch batch) {
  constexpr int BPW = 32 / K;
  __shared__ BlockTab s_tab[WARPS][BPW];
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  build_snap_tables(s_snap5, s_snap6);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, slot = lane / K, k = lane % K;
  const int total = batch.group_end[batch.n - 1];
  for (int gg = blockIdx.x * WARPS + warp; gg < total; gg += gridDim.x * WARPS) {
    int jb = 0;
    while (gg >= batch.group_end[jb]) ++jb;
    const SearchParams &P = batch.P[jb];
    const uint16_t *__restrict__ topk = batch.topk[jb];
    const int nblk = P.bw * P.bh, w2 = 2 * P.sa;
    const uint32_t *prev_hi = reinterpret_cast<const uint32_t *>(P.prev) + 1;
    const int base = (gg - (jb ? batch.group_end[jb - 1] : 0)) * BPW;
    int sumsq = 0;
    if constexpr (BPW == 1) {
      if (base < nblk) {
        const int by = base / P.bw, bx = base - by * P.bw;
        sumsq = stage_block(s_tab[warp][0], P.rgb, P.width, bx, by, lane);
      }
    } else {
      // two blocks per staging pass, half a warp each
#pragma unroll
      for (int jj = 0; jj < BPW; jj += 2) {
        const int ia = base + jj, ib = ia + 1;
        const int ay = ia / P.bw, ax = ia - ay * P.bw, by2 = ib / P.bw, bx2 = ib - by2 * P.bw;
        const int sq = stage_block_pair(s_tab[warp][jj], s_tab[warp][jj + 1], P.rgb, P.width, ax, ay, ia < nblk,
                                        bx2, by2, ib < nblk, lane);
        const int sqa = __shfl_sync(kFull, sq, 0), sqb = __shfl_sync(kFull, sq, 16);
        if (slot == jj) sumsq = sqa;
        if (slot == jj + 1) sumsq = sqb;
      }
    }
    const int idx = base + slot;
    const bool valid = idx < nblk;
    const int by = valid ? idx / P.bw : 0, bx = valid ? idx - by * P.bw : 0;
    const BlockTab &tab = s_tab[warp][slot];
    int e = kInvalid, pos = -1, refit = 0;
    uint32_t cand = 0, eps = 0;
    uint64_t stb = 0;
    if (valid) {
      stb = P.stb[idx];
      const uint16_t p = topk[(size_t)idx * kMaxK + k];
      const int prow = p / w2, pcol = p - prow * w2;
      const int gy = by - P.sa + prow, gx = bx - P.sa + pcol;
      // the scoring kernel lists in-frame window positions only; anything
      // else (a list left from an aborted launch) is ignored, never read
      if (p != kNoProposal && p < w2 * w2 && gy >= 0 && gy < P.bh && gx >= 0 && gx < P.bw) {
        pos = p;
        const size_t nidx = (size_t)gy * P.bw + gx;
        cand = __ldg(prev_hi + 2 * nidx);
        const float4 d = __ldg(P.wdesc + nidx);
        const WeightSums ws{d.x, d.y, d.z, d.w};
        const PixelGroups pg = load_groups(tab);
        e = eval_candidate(tab, pg, s_snap5, s_snap6, cand, ws, (uint32_t)(stb >> 32), P.orig_err[idx], sumsq, eps,
                           refit);
      }
    }
    const int row = pos >= 0 ? pos / w2 : 0;
    // P0: first position with err_diff <= 0
    int k1 = (e != kInvalid && e <= 0) ? pos : 0xFFFF;
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) k1 = min(k1, __shfl_xor_sync(kFull, k1, o));
    const int r0 = k1 < 0xFFFF ? k1 / w2 : 0x7FFF;
    // the last later row with an err_diff < 0, and its first such position
    int k2 = (e != kInvalid && e < 0 && row > r0) ? (row << 16) | (0xFFFF - pos) : 0;
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) k2 = max(k2, __shfl_xor_sync(kFull, k2, o));
    // otherwise the first minimum
    int k3 = e != kInvalid ? ((e + 65536) << 12) | pos : 0x7FFFFFFF;
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) k3 = min(k3, __shfl_xor_sync(kFull, k3, o));
    int sel = -1, m = kInvalid;
    if (k2 > 0) {
      sel = 0xFFFF - (k2 & 0xFFFF);
      m = 0;
    } else if (k1 < 0xFFFF) {
      sel = k1;
      m = 0;
    } else if (k3 != 0x7FFFFFFF) {
      sel = k3 & 0xFFF;
      m = (k3 >> 12) - 65536;
    }
    const bool accept = sel >= 0 && m <= P.thr;
    if (valid && accept && pos == sel) {
      const uint64_t blk = refit ? ((uint64_t)eps | ((uint64_t)cand << 32)) : stb;
      const int col = sel - row * w2;
      P.final_blk[idx] = blk;
      P.motion[idx] = (uint16_t)((col | 0x80) | ((row | 0x80) << 8));
      P.done[idx] = done_word(blk);
    }
    if (valid && !accept && k == 0) {
      P.done[idx] = 0;
      batch.fb_list[jb][atomicAdd(batch.fb_count[jb], 1u)] = (uint32_t)idx;
    }
    __syncwarp();
  }
}

// The exhaustive inter search (InterBlockSearch, codec/dxt_image.cpp:715-774)
// of the listed blocks (sa <= 8), one CTA per block, one window position per
// thread: the short lists of blocks none of whose proposals passed, searched
// side by side so that the kernel ends with its slowest block's 256
// evaluations in parallel rather than a warp's successive rounds. The jobs'
// lists are taken as one concatenated list.
struct ListBatch {
  int n;
  SearchParams P[kMaxBatch];
  const uint32_t *list[kMaxBatch];
  const uint32_t *count[kMaxBatch];
};

template <int THREADS>
__global__ void __launch_bounds__(THREADS) inter_list_kernel(const __grid_constant__ ListBatch batch) {
  static_assert(THREADS >= 256, "one thread per position of a 16x16 window");
  int total = 0;
  for (int j = 0; j < batch.n; ++j) total += (int)__ldcg(batch.count[j]);
  if ((int)blockIdx.x >= total) return;  // the whole CTA, before its barriers
  __shared__ BlockTab s_tab;
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  __shared__ int s_red[2 * (THREADS / 32)];
  __shared__ int s_sumsq;
  build_snap_tables(s_snap5, s_snap6);
  CtaReduce<THREADS> red{s_red, 0};
  for (int k = blockIdx.x; k < total; k += gridDim.x) {
    int jb = 0, off = 0;
    for (;;) {
      const int c = (int)__ldcg(batch.count[jb]);
      if (k - off < c) break;
      off += c;
      ++jb;
    }
    cta_block_search<THREADS>(batch.P[jb], (int)__ldcg(batch.list[jb] + (k - off)), s_tab, s_snap5, s_snap6, red,
                              &s_sumsq);
  }
}

// Exact err_diff (the inter search's refit, validity and error of
// codec/dxt_image.cpp:258-349 against the block's own stb error) of C candidate
// index words for each of B listed blocks: err[b * C + c], INT_MAX when the
// refit would swap the endpoints. One warp per block. Labels the training
// examples of the learned proposal with the exhaustive search's own numbers.
constexpr int kErrWarps = 4;
__global__ void __launch_bounds__(kErrWarps * 32) candidate_errors_kernel(
    const uint8_t *__restrict__ rgb, int width, int bw, const uint64_t *__restrict__ stb,
    const uint32_t *__restrict__ blocks, const uint32_t *__restrict__ cands, int B, int C, int *__restrict__ err) {
  __shared__ BlockTab s_tab[kErrWarps];
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  __shared__ float4 s_wk[4];
  build_snap_tables(s_snap5, s_snap6);
  build_weight_table(s_wk);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = blockIdx.x * kErrWarps + warp; b < B; b += gridDim.x * kErrWarps) {
    const int idx = (int)blocks[b];
    const int by = idx / bw, bx = idx - by * bw;
    const int sumsq = stage_block(s_tab[warp], rgb, width, bx, by, lane);
    const PixelGroups pg = load_groups(s_tab[warp]);
    const uint64_t sb = stb[idx];
    uint32_t px[16];
    load_block_px(rgb, width, bx, by, px);
    const int orig = block_error_physical(px, sb);
    for (int c = lane; c < C; c += 32) {
      const uint32_t cand = cands[(size_t)b * C + c];
      uint32_t eps = 0;
      int refit = 0;
      err[(size_t)b * C + c] = eval_candidate(s_tab[warp], pg, s_snap5, s_snap6, cand, weight_sums(cand, s_wk),
                                              (uint32_t)(sb >> 32), orig, sumsq, eps, refit);
    }
    __syncwarp();
  }
}

}  // namespace mptc
