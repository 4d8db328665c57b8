// Learned candidate proposal: the word dictionary of a frame's final blocks,
// which lets the g network run once per distinct index word.
#pragma once
#include <cstdint>

#include "learned_common.cuh"

namespace mptc {

// ---- word dictionary of a frame ---------------------------------------------------
// A frame's final blocks reuse few distinct index words (1,465-2,026 of
// 129,600 positions on the first frames of the 1080p stream), so g runs once
// per distinct word instead of once per position. word_dict_kernel inserts
// every position's word into an open-addressed table in global memory
// (64-bit entries word << 32 | 1, linear probing, capacity 2^cap_log2 >= 2 x
// positions, zeroed before the launch) and writes the word's table slot to
// rows[pos]; the thread whose insertion creates an entry appends the word and
// its slot to the job's list (*count entries, in no fixed order). g then runs
// over the list and writes the embedding of list entry i to row slots[i] of
// the G table, where the scoring kernel finds it through rows[pos]. The
// embeddings do not depend on the list order. Within a warp, lanes holding the
// same word elect one lane (the lowest) to probe the table.
struct DictArgs {
  const uint32_t *words;  // words[pos * word_stride], pos < n
  int word_stride, n;
  unsigned long long *table;
  int cap_log2;
  uint32_t *rows;                      // n: table slot of the position's word
  uint32_t *list_words, *list_slots;   // the distinct words and their slots
  uint32_t *count;                     // entries in the list
};

// CTAs of job j: [block_end[j - 1], block_end[j]), 256 positions each.
struct DictBatch {
  int n;
  int block_end[kMaxBatch];
  DictArgs a[kMaxBatch];
};

constexpr int kDictThreads = 256;

__global__ void __launch_bounds__(kDictThreads) word_dict_kernel(const __grid_constant__ DictBatch batch) {
  int j = 0;
  while ((int)blockIdx.x >= batch.block_end[j]) ++j;
  const DictArgs &a = batch.a[j];
  const int pos = ((int)blockIdx.x - (j ? batch.block_end[j - 1] : 0)) * kDictThreads + (int)threadIdx.x;
  const bool valid = pos < a.n;
  const uint32_t active = __ballot_sync(0xFFFFFFFFu, valid);
  if (!valid) return;
  const uint32_t word = __ldg(a.words + (size_t)pos * a.word_stride);
  const uint32_t peers = __match_any_sync(active, word);
  const int lane = (int)(threadIdx.x & 31), leader = __ffs(peers) - 1;
  uint32_t slot = 0;
  if (lane == leader) {
    const uint32_t mask = (1u << a.cap_log2) - 1u;
    const unsigned long long entry = ((unsigned long long)word << 32) | 1ull;
    uint32_t h = (word * 0x9E3779B1u) >> (32 - a.cap_log2);
    for (uint32_t it = 0; it <= mask; ++it) {  // the table is never more than half full: it ends
      unsigned long long e = *reinterpret_cast<volatile unsigned long long *>(a.table + h);
      if (e == 0ull) {
        e = atomicCAS(a.table + h, 0ull, entry);
        if (e == 0ull) {
          const uint32_t id = atomicAdd(a.count, 1u);
          a.list_words[id] = word;
          a.list_slots[id] = h;
          break;
        }
      }
      if ((uint32_t)(e >> 32) == word) break;
      h = (h + 1u) & mask;
    }
    slot = h;
  }
  a.rows[pos] = __shfl_sync(active, slot, leader);
}

}  // namespace mptc
