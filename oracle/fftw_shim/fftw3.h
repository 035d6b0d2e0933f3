/*
 * fftw3.h -- project-written stand-in for the subset of the FFTW 3 API that
 * the reference SCFT code uses in its serial (no -DPAR) build.
 *
 * TEST INFRASTRUCTURE ONLY.  This header and fftw_shim.cpp exist so that the
 * reference sources can be compiled into the CPU oracle (oracle/_ref/) on a
 * machine without FFTW.  Nothing in the product library links against it.
 *
 * Symbols the reference needs (code/array_utils.cpp:379-383,
 * code/fft_wrappers.cpp:21,55, code/globals.h:159-167):
 *   fftw_complex, fftw_plan, fftw_malloc, fftw_free, fftw_plan_dft,
 *   fftw_execute, fftw_destroy_plan, FFTW_FORWARD, FFTW_BACKWARD,
 *   FFTW_MEASURE, FFTW_ESTIMATE.
 *
 * Conventions follow FFTW's documented definition of the unnormalised
 * multi-dimensional DFT:  out[k] = sum_j in[j] * exp(sign * 2*pi*i * j.k / n),
 * sign = FFTW_FORWARD (-1) or FFTW_BACKWARD (+1), row-major with the last
 * dimension fastest.  fftw_malloc returns zeroed memory that may be released
 * with free(), because the reference frees some fftw_malloc'd buffers with
 * free() and reads others before writing them (code/1s_update.cpp:73-74).
 */
#ifndef ORACLE_FFTW3_SHIM_H
#define ORACLE_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct oracle_fft_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft(int rank, const int *n, fftw_complex *in,
                        fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif

#endif
