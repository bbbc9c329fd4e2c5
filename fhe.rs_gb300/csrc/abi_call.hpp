// Error translation shared by the C ABI entry points: each runs its body
// through abi_call, which returns FHEG_OK, or maps a library Error to its
// status code, a failed host allocation to FHEG_ERR_BUDGET and any other
// exception to FHEG_ERR_INTERNAL, recording the message for fheg_last_error().
#pragma once

#include <exception>
#include <new>

#include "fheg.h"
#include "lib.hpp"

namespace fheg {

template <class F>
int abi_call(F&& f) {
  try {
    set_last_error("");
    f();
    return FHEG_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return FHEG_ERR_BUDGET;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return FHEG_ERR_INTERNAL;
  }
}

// Argument check of an entry point: FHEG_ERR_INVALID_ARGUMENT with `what`.
inline void abi_need(bool cond, const char* what) {
  if (!cond) throw Error(FHEG_ERR_INVALID_ARGUMENT, what);
}

// Most items one call takes (ciphertexts, polynomials, requests): 2^24.
// Device memory holds far fewer of the smallest items, and below this bound
// no size an entry point derives from the count (count x parts x moduli x
// degree x 8 bytes, with at most 2^33 bytes an item) can wrap around 2^64 to
// a small allocation that the kernels would then overrun.
constexpr size_t kMaxItems = size_t(1) << 24;
inline void abi_count(size_t count) {
  if (count > kMaxItems) throw Error(FHEG_ERR_INVALID_ARGUMENT, "item count above 2^24 per call");
}

}  // namespace fheg
