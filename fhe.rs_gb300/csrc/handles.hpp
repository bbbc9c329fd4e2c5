// Definitions of the opaque handle types of include/fheg.h.
#pragma once

#include <memory>
#include <vector>

#include "fheg.h"
#include "lib.hpp"

struct fheg_context {
  std::shared_ptr<fheg::Context> c;
  // Scratch of fheg_poly_random_from_seed (calls on one context must not overlap).
  std::shared_ptr<fheg::Workspace> ws = std::make_shared<fheg::Workspace>();
};
struct fheg_scaler {
  std::unique_ptr<fheg::Scaler> s;
  fheg::DevBuf scratch;
};
struct fheg_params {
  std::unique_ptr<fheg::Params> p;
  std::vector<fheg_context> level_handles;
  fheg::Workspace ws;  // scratch of the ragged batch entry points
  // Second half of a large ragged rotation batch (api.cu): its stream, fork /
  // join events and scratch.
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  fheg::Workspace side_ws;
  fheg_params() = default;
  fheg_params(const fheg_params&) = delete;
  fheg_params& operator=(const fheg_params&) = delete;
  ~fheg_params() {
    if (side) cudaStreamDestroy(side);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
  }
};
struct fheg_ksk {
  fheg::Ksk k;
};
struct fheg_rgsw {
  fheg::Ksk k;  // count = 2L digits: ksk0's, then ksk1's
};
struct fheg_multiplicator {
  static constexpr int kPipe = 4;  // most streams of the host entry point's copy / compute pipeline
  std::unique_ptr<fheg::Multiplicator> m;
  cudaStream_t pipe[kPipe] = {};      // compute streams
  cudaStream_t copy_in = nullptr;      // every chunk's input copies, in chunk order
  cudaStream_t copy_out = nullptr;     // every chunk's output copy, in chunk order
  fheg::Workspace pipe_ws[kPipe];
  // End of a chunk's input copies / of its multiplication. One event each
  // serves every chunk: each record is waited on right after it is made,
  // and a wait holds the work of the record it follows.
  cudaEvent_t copied = nullptr, computed = nullptr;
  size_t host_chunk = 0;            // pairs per chunk (0 = automatic)
  int host_streams = 3;
  // Second branch of a large direct multiplication (api.cu): its stream,
  // fork / join events and scratch.
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  fheg::Workspace side_ws;
  ~fheg_multiplicator() {
    for (auto& s : pipe)
      if (s) cudaStreamDestroy(s);
    if (copy_in) cudaStreamDestroy(copy_in);
    if (copy_out) cudaStreamDestroy(copy_out);
    if (copied) cudaEventDestroy(copied);
    if (computed) cudaEventDestroy(computed);
    if (side) cudaStreamDestroy(side);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
  }
};
struct fheg_secret_key {
  fheg::SecretKeyDev k;
  mutable fheg::Workspace ws;  // scratch of fheg_decrypt
};

// A key-switching key at the given levels with device room for `count`
// digits; c0 is uploaded from h_c0 unless it is null (api.cu). log_base < 0:
// as KeySwitchingKey::new, a single-modulus key context decomposes in base
// 2^(log2 q / 2) (key_switching_key.rs:70-76); otherwise the base a key
// message names (0 for RNS digits).
fheg_ksk* new_ksk_handle(const fheg_params* par, size_t ciphertext_level, size_t ksk_level, const uint64_t* h_c0,
                         size_t count, int64_t log_base = -1);
