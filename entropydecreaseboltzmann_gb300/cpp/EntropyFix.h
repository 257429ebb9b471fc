// Drop-in replacement for the reference's CalQ/EntropyFix.h.
//
// The same class template EntropyFix<i_type, r_type> (EntropyFix.h:13-46):
// EntropyFix(Nt, eps = 1e-10), EntropyCal, setAverage and FixSol for arrays
// and std::vector, with the reference's latched average and bisection rule;
// the work runs on the GPU through libedb.so.  When the average gets latched
// the reference prints it; so does this header, in the same format.  The
// three-argument FixSol is declared without a definition, as in the
// reference.  Only r_type = double is supported.
#ifndef _ENTROPYFIX_H_
#define _ENTROPYFIX_H_

#include <assert.h>

#include <cmath>
#include <iomanip>
#include <iostream>
#include <type_traits>
#include <vector>

#include "edb_dropin.h"

template <class i_type, class r_type>
class EntropyFix {
  static_assert(std::is_integral<i_type>::value && std::is_same<r_type, double>::value,
                "libedb provides EntropyFix<integer type, double> only");

 private:
  i_type Nt;
  r_type eps;
  edb_efix *h = nullptr;

  EntropyFix() = delete;

  // prints the average when a call latched it (EntropyFix.h:65-78)
  template <class F>
  void latching(F &&call) {
    double avg = 0.0;
    int before = 0, after = 0;
    edb_dropin::check(edb_efix_get_average(h, &avg, &before), "EntropyFix");
    call();
    edb_dropin::check(edb_efix_get_average(h, &avg, &after), "EntropyFix");
    if (!before && after) std::cout << "\nAverafe f\t" << avg << "\n";
  }

 public:
  ~EntropyFix() {
    if (h) edb_efix_destroy(h);
  }
  EntropyFix(i_type _Nt, r_type _eps = 1.0e-10) : Nt(_Nt), eps(_eps) {
    edb_dropin::check(edb_efix_create((int)Nt, eps, &h), "EntropyFix");
  }
  EntropyFix(const EntropyFix &) = delete;
  EntropyFix &operator=(const EntropyFix &) = delete;

  r_type EntropyCal(const std::vector<r_type> &fin) {
    assert((i_type)fin.size() == Nt);
    return EntropyCal((i_type)fin.size(), const_cast<r_type *>(fin.data()));
  }
  r_type EntropyCal(i_type Nf, r_type *fin) {
    double H = 0.0;
    latching([&] { edb_dropin::check(edb_efix_entropy(h, (int)Nf, fin, &H), "EntropyCal"); });
    return H;
  }

  void setAverage(const std::vector<r_type> &fin) {
    assert((i_type)fin.size() == Nt);
    setAverage((i_type)fin.size(), const_cast<r_type *>(fin.data()));
  }
  void setAverage(i_type Nf, r_type *fin) {
    edb_dropin::check(edb_efix_set_average(h, (int)Nf, fin), "setAverage");
    double avg = 0.0;
    int latched = 0;
    edb_dropin::check(edb_efix_get_average(h, &avg, &latched), "setAverage");
    std::cout << "\nAverafe f\t" << avg << "\n";
  }

  void FixSol(std::vector<r_type> &fin, r_type AimEntropy) {
    assert((i_type)fin.size() == Nt);
    FixSol((i_type)fin.size(), fin.data(), AimEntropy);
  }
  void FixSol(i_type Nf, r_type *fin, r_type AimEntropy) {
    latching([&] { edb_dropin::check(edb_efix_fixsol(h, (int)Nf, fin, AimEntropy), "FixSol"); });
  }
  void FixSol(const std::vector<r_type> &fin, std::vector<r_type> &fout, r_type AimEntropy);
};

#endif
