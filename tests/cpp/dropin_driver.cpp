// Reference-style driver compiled against the drop-in headers
// (entropydecreaseboltzmann_gb300/cpp) and linked with libedb.so.
//
//   dropin_driver <in.bin> <out.bin>
// in.bin : int32 N, int32 alpha, int32 filter, then N^3 complex doubles (fin)
//          and N^3 doubles (a positive real array f for EntropyFix)
// out.bin: calQ(fin) (N^3 complex), ifft(fft(fin)) (N^3 complex), fft(fin)
//          (N^3 complex), EntropyCal(f), f after FixSol(f, EntropyCal(f) - 1e-3),
//          funF(0.7, 1.3), filtering(1)
#include <complex>
#include <cstdio>
#include <vector>

#include "EntropyFix.h"
#include "QCalculator.h"
#include "fft3d.h"

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *fi = std::fopen(argv[1], "rb");
  if (!fi) return 3;
  int hdr[3];
  if (std::fread(hdr, sizeof(int), 3, fi) != 3) return 4;
  const int N = hdr[0], alpha = hdr[1], filter = hdr[2];
  const int NQ = N * N * N;
  std::vector<std::complex<double>> fin(NQ), Q(NQ), Fh(NQ), back(NQ);
  std::vector<double> f(NQ);
  if (std::fread(fin.data(), sizeof(double) * 2, NQ, fi) != (size_t)NQ) return 5;
  if (std::fread(f.data(), sizeof(double), NQ, fi) != (size_t)NQ) return 6;
  std::fclose(fi);

  QCalculator<std::complex<double>, double> qc(N, alpha);
  if (!filter) qc.closeFilter();
  qc.genB();
  qc.calQ(Q.data(), fin.data());

  fft3d f3d;
  std::vector<std::complex<double>> tmp(fin);
  f3d.fft(N, N, N, reinterpret_cast<fftw_complex *>(tmp.data()),
          reinterpret_cast<fftw_complex *>(Fh.data()));
  f3d.ifft(N, N, N, reinterpret_cast<fftw_complex *>(back.data()),
           reinterpret_cast<fftw_complex *>(Fh.data()));

  EntropyFix<int, double> ef(NQ);
  const double H = ef.EntropyCal(NQ, f.data());
  ef.FixSol(NQ, f.data(), H - 1e-3);
  const double extra[2] = {qc.funF(0.7, 1.3), qc.filtering(1)};

  FILE *fo = std::fopen(argv[2], "wb");
  if (!fo) return 7;
  std::fwrite(Q.data(), sizeof(double) * 2, NQ, fo);
  std::fwrite(back.data(), sizeof(double) * 2, NQ, fo);
  std::fwrite(Fh.data(), sizeof(double) * 2, NQ, fo);
  std::fwrite(&H, sizeof(double), 1, fo);
  std::fwrite(f.data(), sizeof(double), NQ, fo);
  std::fwrite(extra, sizeof(double), 2, fo);
  std::fclose(fo);
  return 0;
}
