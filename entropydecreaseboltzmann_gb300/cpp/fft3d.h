// Drop-in replacement for the reference's CalQ/fft3d.h.
//
// The same class fft3d with fft(Nx, Ny, Nz, re, fre) and ifft(Nx, Ny, Nz, re,
// fre) (fft3d.h:17-49): unnormalised forward DFT, backward DFT times
// 1/(Nx Ny Nz), computed on the GPU by libedb.so.  FFTW is not needed: when
// <fftw3.h> has not been included, fftw_complex is declared here with FFTW's
// layout (double[2]).
#ifndef __FFT3D_H__
#define __FFT3D_H__

#include <cmath>
#include <complex>

#include "edb_dropin.h"

#ifndef FFTW3_H
typedef double fftw_complex[2];
#endif

class fft3d {
 public:
  fft3d() {}
  ~fft3d() {}

  void fft(int Nx, int Ny, int Nz, fftw_complex *re, fftw_complex *fre) {
    edb_dropin::check(edb_fft3d_fft(Nx, Ny, Nz, reinterpret_cast<const double *>(re),
                                    reinterpret_cast<double *>(fre)),
                      "fft3d::fft");
  }

  void ifft(int Nx, int Ny, int Nz, fftw_complex *re, fftw_complex *fre) {
    edb_dropin::check(edb_fft3d_ifft(Nx, Ny, Nz, reinterpret_cast<double *>(re),
                                     reinterpret_cast<const double *>(fre)),
                      "fft3d::ifft");
  }
};

#endif
