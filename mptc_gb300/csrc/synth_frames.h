/* Seeded synthetic RGB8 frames (integer-exact, identical on every host). */
#ifndef MPTC_SYNTH_FRAMES_H_
#define MPTC_SYNTH_FRAMES_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mptc_synth_config {
  int width, height;            /* pixels */
  int period_min, period_max;   /* sinusoid period range, pixels */
  int amp_min, amp_max;         /* sinusoid amplitude range, 8-bit levels */
  int n_squares, square_size;   /* noise-textured squares and their side, pixels */
  int speed_min, speed_max;     /* square speed range, pixels per frame */
  int cut_every;                /* scene cut (new sinusoids) every N frames; 0 = none */
  uint64_t seed;
} mptc_synth_config;

/* Writes frame `frame` (row-major RGB8, width*height*3 bytes). 0 on success. */
int mptc_synth_frame(const mptc_synth_config *c, int frame, uint8_t *out);
/* Writes `count` consecutive frames starting at `first`. 0 on success. */
int mptc_synth_frames(const mptc_synth_config *c, int first, int count, uint8_t *out);

#ifdef __cplusplus
}
#endif
#endif
