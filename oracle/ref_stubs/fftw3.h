// Stand-in for the FFTW header, only so that the reference's post-processing
// unit compiles for the test oracle, whose r-phi transform does not call it.
// Every function here fails (null plans and buffers).
#ifndef CS_REF_STUB_FFTW3
#define CS_REF_STUB_FFTW3
#include <cstddef>
typedef double fftw_complex[2];
typedef void *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
inline fftw_complex *fftw_alloc_complex(size_t) { return nullptr; }
inline void fftw_free(void *) {}
inline fftw_plan fftw_plan_dft_2d(int, int, fftw_complex *, fftw_complex *, int, unsigned) { return nullptr; }
inline void fftw_execute(const fftw_plan) {}
inline void fftw_destroy_plan(fftw_plan) {}
inline void fftw_cleanup() {}
#endif
