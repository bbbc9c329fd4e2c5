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

}  // namespace fheg
