/* Deterministic synthetic picture-pair generator (host C, identical bytes on x86-64 and aarch64). */
#ifndef QMIV_SYNTH_H
#define QMIV_SYNTH_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct qs_params {
  int32_t  width, height, bitdepth; /* even sizes; 8..14 bits */
  uint32_t seed;                    /* picture seed */
  uint32_t shift_seed;              /* block-shift seed used when drift != 0 */
  int32_t  frame;                   /* temporal index (drift steps every 4 frames) */
  int32_t  drift;                   /* 0: shifts from seed, 1: drifting shifts from shift_seed */
  int32_t  holes;                   /* 1: elliptical holes filled with a constant in the test picture */
  double   noise_sigma;             /* in 8-bit units, scaled by 2^(bd-8) */
  double   offset[3];               /* in 8-bit units, scaled by 2^(bd-8) */
  int32_t  nthreads;
} qs_params;

/* ref/tst: planar 4:2:0, Y (W*H) then Cb, Cr ((W/2)*(H/2) each), uint16 samples */
int qs_generate_pair(const qs_params* p, uint16_t* ref, uint16_t* tst);
/* ref/tst: planar 4:4:4 float in [0,1] (3*W*H) */
int qs_generate_float444(const qs_params* p, float* ref, float* tst, double sigma, double off_range);

#ifdef __cplusplus
}
#endif
#endif
