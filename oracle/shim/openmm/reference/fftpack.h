/* Oracle shim: 3D complex FFT interface used by the Reference PME code.
 * Implemented in oracle/shim_fft.cpp as an unnormalised mixed-radix FFT:
 * FFTPACK_FORWARD uses exp(-2*pi*i*jk/n), FFTPACK_BACKWARD exp(+2*pi*i*jk/n). */
#ifndef MBPOL_SHIM_FFTPACK_H
#define MBPOL_SHIM_FFTPACK_H
struct t_complex {
    double re, im;
    t_complex& operator+=(const t_complex& o) { re += o.re; im += o.im; return *this; }
};
struct fftpack;
typedef struct fftpack* fftpack_t;
enum { FFTPACK_FORWARD = -1, FFTPACK_BACKWARD = 1 };
int fftpack_init_3d(fftpack_t* plan, int nx, int ny, int nz);
int fftpack_exec_3d(fftpack_t plan, int dir, t_complex* in, t_complex* out);
void fftpack_destroy(fftpack_t plan);
#endif
