/* Stand-in for the FFTW3 header, for compiling the reference's own sources
 * into the oracle's reference build (test infrastructure only).  It declares
 * the subset of the FFTW3 API those sources use; fftw_shim.cpp implements it
 * with a project-written double-precision FFT (unnormalised, FFTW's sign
 * convention, row-major with the last dimension contiguous).  Planner flags
 * and wisdom are accepted and ignored. */
#ifndef TDM_REF_FFTW3_SHIM_H
#define TDM_REF_FFTW3_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct tdm_ref_fftw_plan_s* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_WISDOM_ONLY (1U << 21)

void* fftw_malloc(size_t n);
void fftw_free(void* p);
fftw_complex* fftw_alloc_complex(size_t n);
double* fftw_alloc_real(size_t n);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);
void fftw_cleanup(void);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_destroy_plan(fftw_plan p);
int fftw_export_wisdom_to_filename(const char* filename);
int fftw_import_wisdom_from_filename(const char* filename);
int fftw_import_wisdom_from_file(void* file);

#ifdef __cplusplus
}
#endif

#endif
