// Relinearization that allocates no device memory.
//
// Some callers cannot let the library allocate device memory: code that
// records its work into a CUDA stream capture, where a cudaMalloc is not
// capturable and would break the capture; serving loops that must not block
// on the device-wide synchronisation an allocation can cause; and
// applications that hand every byte of device memory to their own pool and
// forbid third-party allocations. fheg_relinearize_noalloc serves them: it
// computes exactly what fheg_relinearize computes, but its scratch lives in a
// fixed, file-scope device array instead of a workspace grown with cudaMalloc.

#include <map>
#include <mutex>
#include <string>

#include "fheg.h"
#include "handles.hpp"
#include "lib.hpp"

namespace {

// 16 MiB of scratch. Every GPU that loads the library holds this array until
// the process exits. Calls on a device share it and it keeps the contents of
// the last call; relinearization overwrites every word it later reads, so
// nothing needs clearing between calls.
constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;
__device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocScratchBytes / sizeof(uint64_t)];

// Device address of g_noalloc_scratch on the current device. In host code the
// array's name is only a host-side stand-in, so the address is looked up
// once per device with cudaGetSymbolAddress (with that device current) and
// cached. The first call of the entry point on a device performs this
// set-up, so that first call should be made before any stream capture.
uint64_t* scratch_on_current_device() {
  static std::mutex mu;
  static std::map<int, uint64_t*> cache;
  int dev = 0;
  fheg::check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess || ptr == nullptr)
    throw fheg::Error(FHEG_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
  cache[dev] = static_cast<uint64_t*>(ptr);
  return cache[dev];
}

}  // namespace

FHEG_API int fheg_relinearize_noalloc(const fheg_ksk* rk, const uint64_t* d_ct3, uint64_t* d_out, size_t count,
                                      void* stream) {
  try {
    fheg::set_last_error("");
    if (!rk || (count && (!d_ct3 || !d_out))) throw fheg::Error(FHEG_ERR_INVALID_ARGUMENT, "null input");
    const fheg::Ksk& k = rk->k;
    const size_t L = k.ctx_ct->L(), Lk = k.ctx_ksk->L(), N = k.ctx_ct->N();
    // Reject by division first, so that a huge count cannot wrap the size
    // computation below around to a small value. A key below the ciphertext
    // level also needs the key context's two output parts and their
    // switched-down copies.
    const size_t per_ct =
        sizeof(uint64_t) * N * (L * (1 + Lk) + (k.switches_down() ? 2 * Lk + 2 * L : 0));
    if (count > kNoAllocScratchBytes / per_ct)
      throw fheg::Error(FHEG_ERR_INVALID_ARGUMENT,
                        "fheg_relinearize_noalloc: " + std::to_string(count) + " ciphertexts need " +
                            std::to_string(per_ct) + " bytes of scratch each; the fixed scratch holds " +
                            std::to_string(kNoAllocScratchBytes) + " bytes");
    // Two regions, each rounded to 256 bytes: the digits of c2, and the key
    // switch's own scratch (their NTTs, plus the switch-down buffers).
    const size_t digit_words = (count * L * N + 31) & ~(size_t)31;
    const size_t d_words = fheg::key_switch_scratch_words(k, count);
    const size_t need = (digit_words + d_words) * sizeof(uint64_t);
    if (need > kNoAllocScratchBytes)
      throw fheg::Error(FHEG_ERR_INVALID_ARGUMENT,
                        "fheg_relinearize_noalloc: " + std::to_string(count) + " ciphertexts need " +
                            std::to_string(need) + " bytes of scratch; the fixed scratch holds " +
                            std::to_string(kNoAllocScratchBytes) + " bytes");
    if (count == 0) return FHEG_OK;
    uint64_t* base = scratch_on_current_device();
    fheg::relinearize_scratch(k, d_ct3, d_out, count, base, base + digit_words, static_cast<cudaStream_t>(stream));
    return FHEG_OK;
  } catch (const fheg::Error& e) {
    fheg::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    fheg::set_last_error(e.what());
    return FHEG_ERR_INTERNAL;
  }
}
