// Drop-in replacement for the reference's CalQ/QCalculator.h.
//
// Same class template, constructor and public methods as the reference
// (QCalculator.h:17-62): QCalculator(N, alpha), closeFilter(), genB(),
// funF(xi, eta), filtering(beta) and the virtual calQ(Qout, fin), with the
// reference's defaults (filter on, kernel scale with 6.62132, its literal
// index loops).  Every method forwards to libedb.so (include/edb.h); the
// table lives on the GPU and calQ runs there.  transf/convertQ, the
// reference's internal layout conversions, have no counterpart.
//
// Only QCalculator<std::complex<double>, double> exists — the reference's only
// instantiation (testBKW3D.cpp:14-15); other types fail to compile because
// there is no CPU path.
#ifndef _QCALCULATOR_H_
#define _QCALCULATOR_H_

#include <assert.h>

#include <cmath>
#include <complex>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <type_traits>
#include <vector>

#include "edb_dropin.h"

template <class c_type, class r_type>
class QCalculator {
  static_assert(std::is_same<c_type, std::complex<double>>::value &&
                    std::is_same<r_type, double>::value,
                "libedb provides QCalculator<std::complex<double>, double> only");

 private:
  int N = 0;
  int NQ = 0;
  int n = 0;      // number of positive exponents
  int alpha = 0;  // 0: Maxwell molecules, 1: hard spheres
  edb_qcalc *h = nullptr;

 public:
  QCalculator() {}
  QCalculator(int _N, int _alpha) : N(_N), alpha(_alpha) { initialize(); }
  virtual ~QCalculator() {
    if (h) edb_qcalc_destroy(h);
  }
  QCalculator(const QCalculator &) = delete;
  QCalculator &operator=(const QCalculator &) = delete;

  void initialize() {
    n = (N - 1) / 2;
    NQ = N * N * N;
    edb_qcalc_desc d;
    edb_dropin::check(edb_qcalc_desc_init(&d, N, alpha), "QCalculator");
    edb_dropin::check(edb_qcalc_create(&d, &h), "QCalculator");
  }

  void closeFilter() { edb_dropin::check(edb_qcalc_close_filter(h), "closeFilter"); }

  void genB() { edb_dropin::check(edb_qcalc_genB(h), "genB"); }

  r_type funF(r_type xi, r_type eta) {
    double out = 0.0;
    edb_dropin::check(edb_funF(alpha, 1, &xi, &eta, &out), "funF");
    return out;
  }

  r_type filtering(int beta) {
    double out = 0.0;
    edb_dropin::check(edb_filtering(N, 1, &beta, &out), "filtering");
    return out;
  }

  // Qout <- Q-hat(fin); fin and Qout hold N^3 complex values in FFTW order.
  virtual void calQ(c_type *Qout, c_type *fin) {
    edb_dropin::check(edb_qcalc_calQ(h, reinterpret_cast<const double *>(fin),
                                     reinterpret_cast<double *>(Qout)),
                      "calQ");
  }
};

#endif
