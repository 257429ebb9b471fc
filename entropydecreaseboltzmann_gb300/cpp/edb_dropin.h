// Shared by the drop-in headers (QCalculator.h, fft3d.h, EntropyFix.h): the
// C ABI of libedb.so and the error policy.  The reference has no error codes
// (it asserts); a failing entry point here throws std::runtime_error with the
// library's message, since silently continuing would hide a missing GPU.
#ifndef EDB_DROPIN_H
#define EDB_DROPIN_H

#include <stdexcept>
#include <string>

#include "edb.h"

namespace edb_dropin {
inline void check(edb_status s, const char *what) {
  if (s != EDB_OK)
    throw std::runtime_error(std::string(what) + ": " + edb_status_string(s) + ": " +
                             edb_last_error());
}
}  // namespace edb_dropin

#endif
