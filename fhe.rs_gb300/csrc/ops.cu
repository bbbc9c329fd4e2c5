// Ring-level operations: contexts, NTTs, element-wise ops, substitution,
// modulus switch-down and RNS scaling (fhe-math `rq`, `ntt`, `rns`).

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include "lib.hpp"
#include "ntt.cuh"

namespace fheg {

std::atomic<uint64_t> g_launches{0};

// Default NTT plan: single pass up to 2^12 (the whole limb in shared memory);
// 2^13 to 2^16 in 2^12-residue blocks, which run three CTAs per SM. At 2^13
// and 2^14 the blocks of a limb form one cluster that exchanges the strided
// stages through distributed shared memory (GB300, 256 x 6 limbs, forward /
// inverse GB/s: 2^13 1,435 / 1,400 against 1,223 / 1,211 in two passes and
// about 1,141 single-pass; 2^14 1,370 / 1,343 against 1,318 / 1,286); at 2^15
// (equal) and 2^16 (1,050 / 958 against 1,166 / 1,135) they run as a strided
// pass plus blocks.
static std::atomic<uint32_t> g_ntt_block[17] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 12, 12, 12, 12};

uint32_t ntt_block_logn(uint32_t logn) { return logn <= 16 ? g_ntt_block[logn].load(std::memory_order_relaxed) : 14; }

// Off by default: on GB300 the hint made the fused tensor NTT 8% slower and
// left the other stages unchanged.
static std::atomic<bool> g_ntt_prefetch{false};
bool ntt_prefetch_enabled() { return g_ntt_prefetch.load(std::memory_order_relaxed); }
void set_ntt_prefetch(bool on) { g_ntt_prefetch.store(on, std::memory_order_relaxed); }

bool ntt_plan_valid(uint32_t logn, uint32_t block_logn) {
  const bool single = block_logn == logn && logn >= 3 && logn <= 14;
  const bool split = logn >= 13 && logn <= 16 && block_logn >= 12 && block_logn <= 14 && block_logn < logn &&
                     logn - block_logn <= 4;
  return single || split;
}

std::vector<uint32_t> ntt_plans(uint32_t logn) {
  std::vector<uint32_t> out;
  for (uint32_t bl = 12; bl <= 14; bl++)
    if (ntt_plan_valid(logn, bl)) out.push_back(bl);
  if (out.empty() && ntt_plan_valid(logn, logn)) out.push_back(logn);
  return out;
}

static std::atomic<bool> g_ntt_cluster[17] = {false, false, false, false, false, false, false, false, false,
                                               false, false, false, false, true,  true,  false, false};
bool ntt_cluster_enabled(uint32_t logn) { return logn <= 16 && g_ntt_cluster[logn].load(std::memory_order_relaxed); }
void set_ntt_cluster(uint32_t logn, bool on) {
  if (logn > 16) throw Error(FHEG_ERR_INVALID_ARGUMENT, "unsupported NTT size");
  g_ntt_cluster[logn].store(on, std::memory_order_relaxed);
}

void set_ntt_block_logn(uint32_t logn, uint32_t block_logn) {
  if (!ntt_plan_valid(logn, block_logn)) throw Error(FHEG_ERR_INVALID_ARGUMENT, "unsupported NTT plan");
  g_ntt_block[logn].store(block_logn, std::memory_order_relaxed);
}

void upload(void* dst, const void* src, size_t bytes) {
  check_cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
}

// ---------------------------------------------------------------------------
// Prime table registry.

std::shared_ptr<PrimeTables> get_prime_tables(uint64_t p, size_t n, uint64_t root) {
  static std::mutex mu;
  static std::map<std::tuple<int, uint64_t, size_t, uint64_t>, std::weak_ptr<PrimeTables>> registry;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (root == 0) root = default_ntt_root(p, n);
  std::lock_guard<std::mutex> lock(mu);
  auto key = std::make_tuple(dev, p, n, root);
  auto it = registry.find(key);
  if (it != registry.end()) {
    if (auto sp = it->second.lock()) return sp;
  }
  auto t = std::make_shared<PrimeTables>();
  t->host = make_ntt_tables(p, n, root);
  t->tables.alloc(4 * n * sizeof(uint64_t));
  std::vector<uint64_t> inter(4 * n);
  for (size_t i = 0; i < n; i++) {
    inter[2 * i] = t->host.omegas[i];
    inter[2 * i + 1] = t->host.omegas_shoup[i];
    inter[2 * n + 2 * i] = t->host.zetas_inv[i];
    inter[2 * n + 2 * i + 1] = t->host.zetas_inv_shoup[i];
  }
  uint64_t* d = t->tables.u64();
  upload(d, inter.data(), 4 * n * 8);
  DevPrime& dp = t->dev;
  dp.p = p;
  dp.p2 = 2 * p;
  barrett128(p, &dp.bhi, &dp.blo);
  dp.ninv = t->host.size_inv;
  dp.ninv_shoup = t->host.size_inv_shoup;
  uint64_t inv = p;  // p^-1 mod 2^64 by Newton's iteration (each step doubles the correct bits)
  for (int k = 0; k < 6; k++) inv *= 2 - p * inv;
  dp.pinv = 0 - inv;
  const uint64_t r_mod_p = (uint64_t)(((unsigned __int128)1 << 64) % p);
  dp.ninv_mont = (uint64_t)((unsigned __int128)dp.ninv * r_mod_p % p);
  dp.ninv_mont_shoup = shoup(dp.ninv_mont, p);
  const uint64_t zlast = t->host.zetas_inv[n - 2];
  dp.zlast_ninv = mulmod(zlast, dp.ninv, p);
  dp.zlast_ninv_shoup = shoup(dp.zlast_ninv, p);
  dp.zlast_ninv_mont = mulmod(zlast, dp.ninv_mont, p);
  dp.zlast_ninv_mont_shoup = shoup(dp.zlast_ninv_mont, p);
  dp.tw = reinterpret_cast<const ulonglong2*>(d);
  dp.itw = reinterpret_cast<const ulonglong2*>(d + 2 * n);
  registry[key] = t;
  return t;
}

// ---------------------------------------------------------------------------
// Context

Context::Context(const std::vector<uint64_t>& m, size_t n, const uint64_t* roots) : degree(n), moduli(m) {
  if (n < 8 || (n & (n - 1))) throw Error(FHEG_ERR_INVALID_ARGUMENT, "The degree is not a power of two larger or equal to 8");
  if (n > (1u << 16)) throw Error(FHEG_ERR_UNSUPPORTED, "degrees above 2^16 are not supported");
  if (m.empty()) throw Error(FHEG_ERR_INVALID_ARGUMENT, "The list of moduli is empty");
  logn = 0;
  while (((size_t)1 << logn) < n) logn++;
  check_cuda(cudaGetDevice(&device), "cudaGetDevice");
  rns.reset(new RnsContextHost(m));
  std::vector<DevPrime> host(m.size());
  for (size_t i = 0; i < m.size(); i++) {
    if (m[i] < 2 || (m[i] >> 62) != 0) throw Error(FHEG_ERR_INVALID_MODULUS, "InvalidModulus");
    primes.push_back(get_prime_tables(m[i], n, roots ? roots[i] : 0));
    host[i] = primes.back()->dev;
  }
  d_primes.alloc(sizeof(DevPrime) * m.size());
  upload(d_primes.ptr, host.data(), sizeof(DevPrime) * m.size());
  // rq/context.rs:66-73 plus the constant of rq/mod.rs:427.
  size_t L = m.size();
  std::vector<uint64_t> sw(3 * (L > 1 ? L - 1 : 1), 0);
  if (L > 1) {
    uint64_t q_last = m[L - 1];
    for (size_t i = 0; i + 1 < L; i++) {
      uint64_t inv = invmod(q_last % m[i], m[i]);
      sw[i] = inv;
      sw[(L - 1) + i] = shoup(inv, m[i]);
      sw[2 * (L - 1) + i] = m[i] - (q_last / 2) % m[i];
    }
  }
  d_switch.alloc(sw.size() * 8);
  upload(d_switch.ptr, sw.data(), sw.size() * 8);
}

std::vector<uint64_t> Context::roots() const {
  std::vector<uint64_t> r;
  for (auto& p : primes) r.push_back(p->host.root);
  return r;
}

std::shared_ptr<Context> Context::prefix(size_t count) const {
  std::vector<uint64_t> m(moduli.begin(), moduli.begin() + count);
  std::vector<uint64_t> r = roots();
  return std::make_shared<Context>(m, degree, r.data());
}

// ---------------------------------------------------------------------------
// NTT on whole contexts.

void ntt_forward(const Context& ctx, PolyRef src, PolyRef dst, uint64_t polys, bool lazy, cudaStream_t st) {
  if (polys == 0) return;
  NttGeom g{ctx.primes_dev(), (uint32_t)ctx.L(), 0};
  if (lazy) ntt_forward_any<false>(ctx.logn, g, polys, SrcPoly{src}, DstPoly{dst}, st);
  else ntt_forward_any<true>(ctx.logn, g, polys, SrcPoly{src}, DstPoly{dst}, st);
}

void ntt_backward(const Context& ctx, PolyRef src, PolyRef dst, uint64_t polys, cudaStream_t st) {
  if (polys == 0) return;
  NttGeom g{ctx.primes_dev(), (uint32_t)ctx.L(), 0};
  ntt_inverse_any(ctx.logn, g, polys, SrcPoly{src}, DstPoly{dst}, st);
}

// ---------------------------------------------------------------------------
// Element-wise kernels. One thread per (poly, limb, coefficient).

__global__ void k_poly_op(const DevPrime* primes, uint32_t limbs, uint32_t logn, int op, PolyRef a, PolyRef b,
                          PolyRef out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  const uint32_t limb = job % limbs;
  const uint32_t poly = job / limbs;
  const DevPrime pr = primes[limb];
  const uint64_t x = a.at(poly, limb)[i];
  uint64_t r;
  if (op == 3) {
    r = x ? pr.p - x : 0;  // zq/mod.rs:175-178 `neg`
  } else {
    const uint64_t y = b.at(poly, limb)[i];
    if (op == 0) r = add_mod(x, y, pr.p);
    else if (op == 1) r = sub_mod(x, y, pr.p);
    else r = mul_mod(x, y, pr);
  }
  out.at(poly, limb)[i] = r;
}

static unsigned blocks_for(uint64_t total, unsigned threads) { return (unsigned)((total + threads - 1) / threads); }

// zq/mod.rs:195-199 `shoup`: floor(x * 2^64 / q) for x < q. With b =
// floor(2^128 / q), t = floor(x * b / 2^64) is that quotient or one less
// (x * (2^128 / q - b) / 2^64 < 1); the remainder x * 2^64 - t q, below 2q,
// tells which.
__device__ __forceinline__ uint64_t shoup_of(uint64_t x, const DevPrime& pr) {
  uint64_t t = x * pr.bhi + __umul64hi(x, pr.blo);
  const uint64_t rem = 0 - t * pr.p;  // x * 2^64 - t q, taken modulo 2^64
  if (rem >= pr.p) t++;
  return t;
}

// Poly::compute_coefficients_shoup (rq/mod.rs:209-223): the Shoup plane of
// NttShoup polynomials.
__global__ void k_poly_shoup(const DevPrime* primes, uint32_t limbs, uint32_t logn, PolyRef a, PolyRef out,
                             uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  const uint32_t limb = job % limbs, poly = job / limbs;
  const DevPrime pr = primes[limb];
  out.at(poly, limb)[i] = shoup_of(a.at(poly, limb)[i], pr);
}

// MulAssign<&Poly<NttShoup>> for Poly<Ntt> (rq/ops.rs:208-245): Shoup
// products with b's companions, reduced (zq/mod.rs:407-416 `mul_shoup_vec`).
__global__ void k_poly_mul_shoup(const DevPrime* primes, uint32_t limbs, uint32_t logn, PolyRef a, PolyRef b,
                                 PolyRef bs, PolyRef out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  const uint32_t limb = job % limbs, poly = job / limbs;
  const uint64_t p = primes[limb].p;
  out.at(poly, limb)[i] = mul_shoup(a.at(poly, limb)[i], b.at(poly, limb)[i], bs.at(poly, limb)[i], p);
}

void poly_compute_shoup(const Context& ctx, PolyRef a, PolyRef out, uint64_t polys, cudaStream_t st) {
  const uint64_t total = polys * ctx.L() << ctx.logn;
  if (total == 0) return;
  k_poly_shoup<<<blocks_for(total, 256), 256, 0, st>>>(ctx.primes_dev(), (uint32_t)ctx.L(), ctx.logn, a, out, total);
  after_launch("k_poly_shoup");
}

void poly_mul_shoup(const Context& ctx, PolyRef a, PolyRef b, PolyRef bs, PolyRef out, uint64_t polys,
                    cudaStream_t st) {
  const uint64_t total = polys * ctx.L() << ctx.logn;
  if (total == 0) return;
  k_poly_mul_shoup<<<blocks_for(total, 256), 256, 0, st>>>(ctx.primes_dev(), (uint32_t)ctx.L(), ctx.logn, a, b, bs,
                                                           out, total);
  after_launch("k_poly_mul_shoup");
}

void poly_op(const Context& ctx, int op, PolyRef a, PolyRef b, PolyRef out, uint64_t polys, cudaStream_t st) {
  uint64_t total = polys * ctx.L() << ctx.logn;
  if (total == 0) return;
  k_poly_op<<<blocks_for(total, 256), 256, 0, st>>>(ctx.primes_dev(), (uint32_t)ctx.L(), ctx.logn, op, a, b, out,
                                                    total);
  after_launch("k_poly_op");
}

// MulAssign<&BigUint> for Poly (rq/ops.rs:297-352): every limb times the
// scalar's projection s_j = scalar mod q_j, as zq `scalar_mul_vec`
// (zq/mod.rs:349-355: Shoup products, reduced). Any representation.
struct ScalarLimbs {
  ulonglong2 s[kMaxScalarLimbs];  // (s_j, shoup(s_j))
};

__global__ void k_poly_scalar_mul(const DevPrime* primes, uint32_t limbs, uint32_t logn,
                                  const __grid_constant__ ScalarLimbs sc, PolyRef in, PolyRef out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  const uint32_t limb = job % limbs;
  const uint32_t poly = job / limbs;
  const uint64_t p = primes[limb].p;
  out.at(poly, limb)[i] = mul_shoup(in.at(poly, limb)[i], sc.s[limb].x, sc.s[limb].y, p);
}

void poly_scalar_mul(const Context& ctx, const BigUint& scalar, PolyRef in, PolyRef out, uint64_t polys,
                     cudaStream_t st) {
  if (ctx.L() > kMaxScalarLimbs) throw Error(FHEG_ERR_UNSUPPORTED, "scalar multiplication supports up to 64 moduli");
  ScalarLimbs sc;
  memset(&sc, 0, sizeof(sc));
  for (size_t j = 0; j < ctx.L(); j++) {
    const uint64_t q = ctx.moduli[j];
    const uint64_t v = scalar.mod_u64(q);
    sc.s[j] = make_ulonglong2(v, shoup(v, q));
  }
  const uint64_t total = polys * ctx.L() << ctx.logn;
  if (total == 0) return;
  k_poly_scalar_mul<<<blocks_for(total, 256), 256, 0, st>>>(ctx.primes_dev(), (uint32_t)ctx.L(), ctx.logn, sc, in,
                                                            out, total);
  after_launch("k_poly_scalar_mul");
}

// Poly::substitute (rq/mod.rs:319-369).
//  Ntt:        q[bitrev[j]] = p[power_bitrev[j]], power_bitrev[j] =
//              bitrev(((e-1)/2 + j*e) mod N): output i reads input g(i)
//              with g(i) = bitrev(((e-1)/2 + bitrev(i)*e) mod N).
//  PowerBasis: coefficient j moves to (j*e) mod N, negated when
//              (j*e) mod 2N >= N.
__device__ __forceinline__ uint32_t brev(uint32_t x, uint32_t logn) { return __brev(x) >> (32 - logn); }

__device__ __forceinline__ uint32_t subst_gather(uint32_t i, uint64_t e, uint32_t logn) {
  const uint64_t mask = (1ull << logn) - 1;
  const uint64_t power = (((e - 1) >> 1) + (uint64_t)brev(i, logn) * e) & mask;
  return brev((uint32_t)power, logn);
}

__global__ void k_substitute(const DevPrime* primes, uint32_t limbs, uint32_t logn, uint64_t e, int ntt, PolyRef in,
                             PolyRef out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  const uint32_t limb = job % limbs;
  const uint32_t poly = job / limbs;
  if (ntt) {
    out.at(poly, limb)[i] = in.at(poly, limb)[subst_gather(i, e, logn)];
  } else {
    const uint64_t n = 1ull << logn;
    const uint64_t pw = ((uint64_t)i * e) & (2 * n - 1);
    const uint64_t v = in.at(poly, limb)[i];
    const uint64_t p = primes[limb].p;
    out.at(poly, limb)[pw & (n - 1)] = (pw & n) ? (v ? p - v : 0) : v;
  }
}

void poly_substitute(const Context& ctx, uint64_t exponent, bool ntt, PolyRef in, PolyRef out, uint64_t polys,
                     cudaStream_t st) {
  uint64_t e = exponent % (2 * ctx.N());
  if ((e & 1) == 0) throw Error(FHEG_ERR_INVALID_ARGUMENT, "The exponent should be odd modulo 2 * degree");
  uint64_t total = polys * ctx.L() << ctx.logn;
  if (total == 0) return;
  k_substitute<<<blocks_for(total, 256), 256, 0, st>>>(ctx.primes_dev(), (uint32_t)ctx.L(), ctx.logn, e, ntt ? 1 : 0,
                                                       in, out, total);
  after_launch("k_substitute");
}

// ---------------------------------------------------------------------------
// Modulus switch-down (rq/mod.rs:390-448) of coefficient i of limb `limb`,
// given the power-basis residues x_i (mod q_i) and x_L (mod q_last).
struct SwitchConsts {
  const uint64_t* sw;  // inv[L-1], inv_shoup[L-1], (q_i - (q_last/2 mod q_i))[L-1]
  uint64_t q_last;
  uint32_t lm1;  // L - 1
};

__device__ __forceinline__ uint64_t switch_down_value(const SwitchConsts& c, uint32_t limb, const DevPrime& pr,
                                                      uint64_t xi, uint64_t xl) {
  const uint64_t last = reduce_once(xl + (c.q_last >> 1), c.q_last);  // rq/mod.rs:417-419
  const uint64_t tmp = reduce64_lazy(last, pr) + __ldg(c.sw + 2 * c.lm1 + limb);  // rq/mod.rs:430
  const uint64_t coeff = xi + 3 * pr.p - tmp;                                     // rq/mod.rs:434
  return mul_shoup(coeff, __ldg(c.sw + limb), __ldg(c.sw + c.lm1 + limb), pr.p);  // rq/mod.rs:437
}

__global__ void k_switch_down_pb(const DevPrime* primes, SwitchConsts c, uint32_t logn, PolyRef in, PolyRef out,
                                 uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  const uint32_t limb = job % c.lm1;
  const uint32_t poly = job / c.lm1;
  const DevPrime pr = primes[limb];
  out.at(poly, limb)[i] = switch_down_value(c, limb, pr, in.at(poly, limb)[i], in.at(poly, c.lm1)[i]);
}

static SwitchConsts switch_consts(const Context& ctx) {
  if (ctx.L() < 2) throw Error(FHEG_ERR_NO_MORE_CONTEXT, "NoMoreContext");
  SwitchConsts c;
  c.sw = ctx.d_switch.u64();
  c.q_last = ctx.moduli.back();
  c.lm1 = (uint32_t)(ctx.L() - 1);
  return c;
}

void poly_switch_down_pb(const Context& ctx, PolyRef in, PolyRef out, uint64_t polys, cudaStream_t st) {
  SwitchConsts c = switch_consts(ctx);
  uint64_t total = polys * c.lm1 << ctx.logn;
  if (total == 0) return;
  k_switch_down_pb<<<blocks_for(total, 256), 256, 0, st>>>(ctx.primes_dev(), c, ctx.logn, in, out, total);
  after_launch("k_switch_down_pb");
}

// Forward-NTT source that performs the switch-down on the fly from a
// power-basis batch: fuses rq/mod.rs:390-448 into the next `into_ntt`.
struct SrcSwitchDown {
  PolyRef pb;
  SwitchConsts c;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    return switch_down_value(c, j.limb, pr, pb.at(j.poly, j.limb)[i], pb.at(j.poly, c.lm1)[i]);
  }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const {
    prefetch_l2(pb.at(j.poly, j.limb) + i);
    prefetch_l2(pb.at(j.poly, c.lm1) + i);
  }
};

void poly_switch_down_ntt(const Context& ctx, PolyRef in, PolyRef out, uint64_t polys, cudaStream_t st) {
  SwitchConsts c = switch_consts(ctx);
  if (polys == 0) return;
  ntt_backward(ctx, in, in, polys, st);
  NttGeom g{ctx.primes_dev(), c.lm1, 0};
  ntt_forward_any<true>(ctx.logn, g, polys, SrcSwitchDown{in, c}, DstPoly{out}, st);
}

// ---------------------------------------------------------------------------
// RNS scaling (rns/scaler.rs:249-352), one thread per coefficient.
//
// The reference accumulates in wrapping 256-bit integers; the sums here are
// the same integers accumulated exactly in 32-bit words:
//   G = sum_k r_k * theta_garner_k           (< 2^192 by the choice of shift)
//   O = sum_k (+/-) r_k * theta_omega_k - (+/-) v * theta_gamma   (mod 2^256)
// and each output residue is one exact dot product reduced once:
//   y_j = sum_k r_k * omega_jk + v_j * (q_j - gamma_j) + w_term  (mod q_j),
// which equals the reference's lazily reduced sum modulo q_j.

__device__ __forceinline__ uint64_t join(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }

// Low 128 bits of (w >> s) for an nw-word little-endian value (32-bit words).
__device__ __forceinline__ void shr_words(const uint32_t* w, int nw, uint32_t s, uint64_t* lo, uint64_t* hi) {
  uint32_t o[4];
  const uint32_t ws = s >> 5, bs = s & 31;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const uint32_t idx = ws + k;
    uint32_t a = 0, b = 0;
#pragma unroll
    for (int m = 0; m < 8; m++) {
      if (m < nw && (uint32_t)m == idx) a = w[m];
      if (m < nw && (uint32_t)m == idx + 1) b = w[m];
    }
    o[k] = bs ? ((a >> bs) | (b << (32 - bs))) : a;
  }
  *lo = join(o[0], o[1]);
  *hi = join(o[2], o[3]);
}

// 256-bit a += b, a -= b (32-bit words).
__device__ __forceinline__ void add256w(uint32_t* a, const uint32_t* b) {
  asm("add.cc.u32 %0, %0, %8;\n\taddc.cc.u32 %1, %1, %9;\n\taddc.cc.u32 %2, %2, %10;\n\taddc.cc.u32 %3, %3, %11;\n\t"
      "addc.cc.u32 %4, %4, %12;\n\taddc.cc.u32 %5, %5, %13;\n\taddc.cc.u32 %6, %6, %14;\n\taddc.u32 %7, %7, %15;"
      : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
      : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
}

__device__ __forceinline__ void sub256w(uint32_t* a, const uint32_t* b) {
  asm("sub.cc.u32 %0, %0, %8;\n\tsubc.cc.u32 %1, %1, %9;\n\tsubc.cc.u32 %2, %2, %10;\n\tsubc.cc.u32 %3, %3, %11;\n\t"
      "subc.cc.u32 %4, %4, %12;\n\tsubc.cc.u32 %5, %5, %13;\n\tsubc.cc.u32 %6, %6, %14;\n\tsubc.u32 %7, %7, %15;"
      : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
      : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
}

// High parts of the scaler's sums. The sums only matter at bit 96 and above
// (v needs G >> (shift - 1) with shift >= 123, w needs S >> 126), so the
// fast path adds only the partial products x_i b_j (32-bit words) that
// reach word 3: those with i + j >= 3, and the high halves of those with
// i + j = 2. The rest of a term x * b (x < 2^64, b < 2^128) is below
// 2^64 + 4 * 2^96 < 5 * 2^96, so a sum of F such terms is its kept part (a
// multiple of 2^96) plus less than 5F * 2^96; a result whose kept part is
// that close to a rounding boundary is recomputed exactly.
//
// h[0..NH) are words 3 .. 2 + NH of the sum: NH = 3 for a sum below 2^192,
// NH = 5 for a sum taken modulo 2^256.
template <int NH>
__device__ __forceinline__ void mac_hi(uint32_t* h, uint64_t x, uint64_t blo, uint64_t bhi) {
  static_assert(NH == 3 || NH == 5, "three or five high words");
  if constexpr (NH == 3) {
    asm("{\n\t"
        ".reg .u32 x0, x1, b0, b1, b2, b3;\n\t"
        "mov.b64 {x0, x1}, %3;\n\t"
        "mov.b64 {b0, b1}, %4;\n\t"
        "mov.b64 {b2, b3}, %5;\n\t"
        "mad.hi.cc.u32 %0, x0, b2, %0;\n\t"
        "madc.hi.cc.u32 %1, x0, b3, %1;\n\t"
        "madc.hi.u32 %2, x1, b3, %2;\n\t"
        "mad.lo.cc.u32 %0, x0, b3, %0;\n\t"
        "madc.lo.cc.u32 %1, x1, b3, %1;\n\t"
        "addc.u32 %2, %2, 0;\n\t"
        "mad.hi.cc.u32 %0, x1, b1, %0;\n\t"
        "madc.hi.cc.u32 %1, x1, b2, %1;\n\t"
        "addc.u32 %2, %2, 0;\n\t"
        "mad.lo.cc.u32 %0, x1, b2, %0;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.u32 %2, %2, 0;\n\t"
        "}"
        : "+r"(h[0]), "+r"(h[1]), "+r"(h[2])
        : "l"(x), "l"(blo), "l"(bhi));
  } else {
    asm("{\n\t"
        ".reg .u32 x0, x1, b0, b1, b2, b3;\n\t"
        "mov.b64 {x0, x1}, %5;\n\t"
        "mov.b64 {b0, b1}, %6;\n\t"
        "mov.b64 {b2, b3}, %7;\n\t"
        "mad.hi.cc.u32 %0, x0, b2, %0;\n\t"
        "madc.hi.cc.u32 %1, x0, b3, %1;\n\t"
        "madc.hi.cc.u32 %2, x1, b3, %2;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.lo.cc.u32 %0, x0, b3, %0;\n\t"
        "madc.lo.cc.u32 %1, x1, b3, %1;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.hi.cc.u32 %0, x1, b1, %0;\n\t"
        "madc.hi.cc.u32 %1, x1, b2, %1;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.lo.cc.u32 %0, x1, b2, %0;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "}"
        : "+r"(h[0]), "+r"(h[1]), "+r"(h[2]), "+r"(h[3]), "+r"(h[4])
        : "l"(x), "l"(blo), "l"(bhi));
  }
}

// Words 3..7 of v * theta_gamma for v < 2^96 (vlo, vhi, vhi < 2^32), kept
// as in mac_hi: the low 64 bits of v through mac_hi (dropping less than
// 5 * 2^96), the third word's partial products at word 2 and above (dropping
// the low half of its lowest one, less than 2^96).
__device__ __forceinline__ void mul_v_hi(uint32_t* h, uint64_t vlo, uint64_t vhi, uint64_t blo, uint64_t bhi) {
#pragma unroll
  for (int k = 0; k < 5; k++) h[k] = 0;
  mac_hi<5>(h, vlo, blo, bhi);
  asm("{\n\t"
      ".reg .u32 v2, b0, b1, b2, b3;\n\t"
      "cvt.u32.u64 v2, %5;\n\t"
      "mov.b64 {b0, b1}, %6;\n\t"
      "mov.b64 {b2, b3}, %7;\n\t"
      "mad.hi.cc.u32 %0, v2, b0, %0;\n\t"
      "madc.hi.cc.u32 %1, v2, b1, %1;\n\t"
      "madc.hi.cc.u32 %2, v2, b2, %2;\n\t"
      "madc.hi.cc.u32 %3, v2, b3, %3;\n\t"
      "addc.u32 %4, %4, 0;\n\t"
      "mad.lo.cc.u32 %0, v2, b1, %0;\n\t"
      "madc.lo.cc.u32 %1, v2, b2, %1;\n\t"
      "madc.lo.cc.u32 %2, v2, b3, %2;\n\t"
      "addc.cc.u32 %3, %3, 0;\n\t"
      "addc.u32 %4, %4, 0;\n\t"
      "}"
      : "+r"(h[0]), "+r"(h[1]), "+r"(h[2]), "+r"(h[3]), "+r"(h[4])
      : "l"(vhi), "l"(blo), "l"(bhi));
}

// 160-bit a += b, a -= b (32-bit words).
__device__ __forceinline__ void add160w(uint32_t* a, const uint32_t* b) {
  asm("add.cc.u32 %0, %0, %5;\n\taddc.cc.u32 %1, %1, %6;\n\taddc.cc.u32 %2, %2, %7;\n\taddc.cc.u32 %3, %3, %8;\n\t"
      "addc.u32 %4, %4, %9;"
      : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4])
      : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]));
}

__device__ __forceinline__ void sub160w(uint32_t* a, const uint32_t* b) {
  asm("sub.cc.u32 %0, %0, %5;\n\tsubc.cc.u32 %1, %1, %6;\n\tsubc.cc.u32 %2, %2, %7;\n\tsubc.cc.u32 %3, %3, %8;\n\t"
      "subc.u32 %4, %4, %9;"
      : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4])
      : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]));
}

// Full 128 x 128 -> 256-bit product (32-bit words).
__device__ __forceinline__ void mul128x128w(uint32_t* r, uint64_t alo, uint64_t ahi, uint64_t blo, uint64_t bhi) {
#pragma unroll
  for (int k = 0; k < 8; k++) r[k] = 0;
  uint32_t t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  mac256(t, alo, blo, bhi);  // alo * b at word 0
  uint32_t hi6[6] = {0, 0, 0, 0, 0, 0};
  mac192(hi6, ahi, blo, bhi);  // ahi * b at word 2 (< 2^192)
  uint32_t u[8] = {0, 0, hi6[0], hi6[1], hi6[2], hi6[3], hi6[4], hi6[5]};
  add256w(t, u);
#pragma unroll
  for (int k = 0; k < 8; k++) r[k] = t[k];
}

// All constants of one launch travel in the kernel's parameter space, so
// every multiply-add reads its constant operand straight from the constant
// bank (fully unrolled loops give compile-time offsets). Outputs are limbs
// start .. start + out_len of the target; the rows of omega, gamma and the
// primes are pre-sliced on the host so output o uses row o.
//
// Kernels with an exact source count (EXACT) take odd target moduli, with
// omega, gamma_neg and gamma_neg_hi in Montgomery form (times 2^64 mod q_j):
// the exact sum S is then 2^64 times the output's sum, and one Montgomery
// step divides it back out (mont_fold), with about a third of the multiplies
// of a 128-bit Barrett reduction. The generic kernels take plain constants
// and reduce S by Barrett (any moduli).
template <int MAXF, int MAXT>
struct RnsLaunch {
  uint32_t from_len, out_len, is_one, shift;
  uint32_t tg_sign, to_sign;  // to_sign: bit k = sign of theta_omega_k
  uint64_t tg_lo, tg_hi;
  uint64_t tgar_lo[MAXF], tgar_hi[MAXF];
  uint64_t to_lo[MAXF], to_hi[MAXF];
  uint64_t omega[MAXT][MAXF];
  uint64_t gamma_neg[MAXT];     // (q_j - gamma_j) mod q_j
  uint64_t gamma_neg_hi[MAXT];  // gamma_neg * 2^62 mod q_j
  uint64_t p[MAXT], bhi[MAXT], blo[MAXT];
  uint64_t pinv[MAXT];  // -q_j^-1 mod 2^64 (EXACT)
  // w mod q_j as whi * (2^64 mod q_j) + wlo (EXACT): the Shoup companions of
  // 2^64 mod q_j and of 1, and wbig = every q_j above 2^61 (wlo < 8 q_j).
  uint32_t wbig;
  uint64_t r64[MAXT], r64_shoup[MAXT], one_shoup[MAXT];
};


// EXACT: the source count is MAXF itself (a compile-time constant), so the
// unrolled loops carry no predicated-off terms; used for the counts the
// default multiplications produce (L and 2L + 1 source moduli).
//
// TOP > 0: `in` holds the block pass of a two-pass inverse NTT whose last TOP
// strided stages and final scale have not run. Each CTA of 128 threads then
// owns the 128 coefficients b + t * 2^(logn - TOP) of 128 >> TOP groups b
// (t < 2^TOP); it applies those stages to every source limb of its groups
// (inv_top_stages, the strided inverse pass's arithmetic) into shared memory,
// and each thread scales one coefficient from there. The strided pass and
// its round trip through HBM disappear; the results are the same.
//
// With TOP > 0 and fwd_primes set, the outputs are themselves the input of a
// two-pass forward NTT whose strided first TOP stages this kernel applies
// (fwd_top_stages, output limb o in fwd_primes[o]): they go through shared
// memory so that each group's 2^TOP coefficients meet, and leave lazy in
// [0, 4p) for the block pass.
template <int WORDS>
__device__ __forceinline__ uint64_t* rns_stage_buffer() {
  __shared__ uint64_t buf[WORDS];
  return buf;
}

// Forward stages of the kernel's epilogue (ForwardTop for one launch; primes
// null: none).
struct FwdEpilogue {
  const DevPrime* primes;
  uint32_t period, take;
  const DevPrime* digit_primes;
  uint32_t digit_limbs, digit_raw;
  PolyRef digits;
};

// The exact sums of the rare coefficients whose fast high-word sums sit next
// to a rounding boundary, kept out of line so that the hot kernel body stays
// small in the instruction cache: G (six words) and S (eight words, mod
// 2^256) as the reference accumulates them.
template <int MAXF, int MAXT>
__device__ __noinline__ void rns_exact_g(const RnsLaunch<MAXF, MAXT>* s, const uint64_t* r, uint32_t F, uint32_t* g) {
#pragma unroll 1
  for (int k = 0; k < 6; k++) g[k] = 0;
#pragma unroll 1
  for (uint32_t k = 0; k < F; k++) mac192(g, r[k], s->tgar_lo[k], s->tgar_hi[k]);
}

template <int MAXF, int MAXT>
__device__ __noinline__ void rns_exact_s(const RnsLaunch<MAXF, MAXT>* s, const uint64_t* r, uint32_t F, uint64_t vlo,
                                        uint64_t vhi, uint32_t* pos) {
  uint32_t neg[8];
#pragma unroll 1
  for (int k = 0; k < 8; k++) pos[k] = neg[k] = 0;
#pragma unroll 1
  for (uint32_t k = 0; k < F; k++) {
    if ((s->to_sign >> k) & 1) mac256(neg, r[k], s->to_lo[k], s->to_hi[k]);
    else mac256(pos, r[k], s->to_lo[k], s->to_hi[k]);
  }
  sub256w(pos, neg);
  uint32_t vt[8];
  mul128x128w(vt, vlo, vhi, s->tg_lo, s->tg_hi);
  if (s->tg_sign) add256w(pos, vt);
  else sub256w(pos, vt);
}

template <int MAXF, int MAXT, bool EXACT, int TOP>
__global__ void __launch_bounds__(128) k_rns_scale(const __grid_constant__ RnsLaunch<MAXF, MAXT> s, uint32_t logn,
                                                   PolyRef in, PolyRef out, uint64_t total,
                                                   const DevPrime* src_primes, uint32_t src_mont,
                                                   const FwdEpilogue fe) {
  const uint32_t F = EXACT ? (uint32_t)MAXF : s.from_len;
  constexpr int G = 128 >> TOP;  // groups per CTA (TOP > 0)
  uint32_t i, poly, b0 = 0, logb = 0, t = 0, gi = 0;
  bool fwd_here = false, dig_here = false;  // uniform across the CTA (one polynomial)
  uint64_t r[MAXF];
  if constexpr (TOP == 0) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= total) return;
    i = gid & ((1u << logn) - 1);
    poly = (uint32_t)(gid >> logn);
    const uint64_t* src = in.at(poly, 0) + i;
#pragma unroll
    for (int k = 0; k < MAXF; k++) r[k] = k < (int)F ? src[(uint64_t)k << logn] : 0;
  } else {
    // The grid covers whole polynomials (2^logn is a multiple of 128), so
    // every thread reaches the barriers.
    uint64_t* staged = rns_stage_buffer<(MAXF > MAXT ? MAXF : MAXT) * 128>();
    poly = blockIdx.x >> (logn - 7);
    b0 = (blockIdx.x & ((1u << (logn - 7)) - 1)) * G;
    logb = logn - TOP;
    for (uint32_t item = threadIdx.x; item < F * G; item += 128) {
      const uint32_t k = item / G, gi = item % G;
      const uint64_t* row = in.at(poly, k) + b0 + gi;
      uint64_t x[1 << TOP];
#pragma unroll
      for (int t = 0; t < (1 << TOP); t++) x[t] = row[(uint64_t)t << logb];
      inv_top_stages<TOP>(x, src_primes[k], 1u << logn, src_mont != 0);
#pragma unroll
      for (int t = 0; t < (1 << TOP); t++) staged[(k * (1 << TOP) + t) * G + gi] = x[t];
    }
    __syncthreads();
    t = threadIdx.x / G;
    gi = threadIdx.x % G;
    i = b0 + gi + (t << logb);
#pragma unroll
    for (int k = 0; k < MAXF; k++) r[k] = k < (int)F ? staged[(k * (1 << TOP) + t) * G + gi] : 0;
    if (fe.primes) {
      const uint32_t part = fe.period ? poly % fe.period : 0;
      fwd_here = part < fe.take;
      dig_here = !fwd_here && fe.digit_primes != nullptr;
    }
    if (fwd_here || dig_here) __syncthreads();  // the buffer takes the outputs next
  }

  // scaler.rs:260-272: v = ceil((G >> (shift - 1)) / 2). Fast path: the
  // kept high words of G; exact when G >> (shift - 1) cannot change under
  // the dropped part (below 5F * 2^96): (H mod 2^e) + 5F < 2^e, e = shift - 97.
  uint32_t g[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int k = 0; k < MAXF; k++)
    if (k < (int)F) mac_hi<3>(g + 3, r[k], s.tgar_lo[k], s.tgar_hi[k]);
  // shift >= 122 for any source count up to 128 moduli below 2^62; smaller
  // shifts (never produced) take the exact path.
  const uint32_t e_bits = s.shift >= 104 ? s.shift - 97 : 7;
  bool exact = s.shift < 104 || (g[3] & ((1u << e_bits) - 1)) >= (1u << e_bits) - 5 * F;
  if (exact) rns_exact_g<MAXF, MAXT>(&s, r, F, g);
  uint64_t vlo, vhi;
  shr_words(g, 6, s.shift - 1, &vlo, &vhi);
  {
    const uint64_t odd = vlo & 1;
    vlo = (vlo >> 1) | (vhi << 63);
    vhi >>= 1;
    vlo += odd;
    vhi += (vlo < odd);
  }

  // scaler.rs:276-314. Fast path: the kept high words of the signed sum S
  // (the dropped part lies in (-(5F + 6), 5F + 6) * 2^96: 5 * 2^96 per term
  // and 6 * 2^96 for v * theta_gamma); exact when S >> 126 cannot change,
  // i.e. H mod 2^30 is at least 5F + 6 away from a multiple of 2^30.
  bool w_sign = false;
  uint64_t wlo = 0, whi = 0;
  if (!s.is_one) {
    uint32_t pos[8] = {0, 0, 0, 0, 0, 0, 0, 0}, neg[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (!exact) {
#pragma unroll
      for (int k = 0; k < MAXF; k++) {
        if (k < (int)F) {
          if ((s.to_sign >> k) & 1) mac_hi<5>(neg + 3, r[k], s.to_lo[k], s.to_hi[k]);
          else mac_hi<5>(pos + 3, r[k], s.to_lo[k], s.to_hi[k]);
        }
      }
      sub160w(pos + 3, neg + 3);
      uint32_t vt[5];
      mul_v_hi(vt, vlo, vhi, s.tg_lo, s.tg_hi);
      if (s.tg_sign) add160w(pos + 3, vt);
      else sub160w(pos + 3, vt);
      const uint32_t m = pos[3] & ((1u << 30) - 1), margin = 5 * F + 6;
      exact = m < margin || m > (1u << 30) - 1 - margin;
    }
    if (exact) rns_exact_s<MAXF, MAXT>(&s, r, F, vlo, vhi, pos);
    w_sign = (pos[7] >> 31) != 0;
    if (w_sign) {
      uint32_t nw[8];
#pragma unroll
      for (int k = 0; k < 8; k++) nw[k] = ~pos[k];
      shr_words(nw, 8, 126, &wlo, &whi);
      wlo += 1;
      whi += (wlo == 0);
      wlo = (wlo >> 1) | (whi << 63);
      whi >>= 1;
    } else {
      shr_words(pos, 8, 126, &wlo, &whi);
      const uint64_t odd = wlo & 1;
      wlo = (wlo >> 1) | (whi << 63);
      whi >>= 1;
      wlo += odd;
      whi += (wlo < odd);
    }
  }

  // scaler.rs:316-351. Above 8 source moduli the output loop stays
  // rolled: unrolling it as well made the kernel body overflow the
  // instruction cache (ncu: a third of the stall cycles waiting for
  // instructions); its constants are then read with an indexed constant-bank
  // load per term. Smaller bodies run faster unrolled.
  constexpr int kOutUnroll = MAXF > 8 ? 1 : MAXT;
  // v <= 32 * 2^62 (at most 32 sources, each residue below 2^62), so
  // v * gamma = (v mod 2^62) * gamma + (v >> 62) * (gamma * 2^62 mod q_j):
  // two exact terms of the 128-bit sum below, and v needs no reduction
  // modulo each q_j. The sum then holds at most 15 terms below 2^124 (and a
  // few small ones) between reductions: below 2^128.
  const uint64_t v_low = vlo & ((1ull << 62) - 1);
  const uint64_t v_top = (vlo >> 62) | (vhi << 2);
  uint64_t* dst = out.at(poly, 0) + i;
#pragma unroll kOutUnroll
  for (int o = 0; o < MAXT; o++) {
    if (o < (int)s.out_len) {
      DevPrime pr;
      pr.p = s.p[o];
      pr.p2 = 2 * s.p[o];
      pr.bhi = s.bhi[o];
      pr.blo = s.blo[o];
      uint64_t y;
      if constexpr (EXACT) {
        // Every term below 2^62 q_j (r_k, v_low < 2^62; v_top < 32), so 14
        // products and the two gamma terms keep hi below 4 q_j.
        uint64_t lo = 0, hi = 0, acc = 0;
        mac128(hi, lo, v_low, s.gamma_neg[o]);
        mac128(hi, lo, v_top, s.gamma_neg_hi[o]);
#pragma unroll
        for (int k = 0; k < MAXF; k++) {
          if (k < (int)F) {
            mac128(hi, lo, r[k], s.omega[o][k]);
            if ((k % 14) == 13) {
              acc = csub(acc + mont_fold(hi, lo, pr.p, s.pinv[o]), pr.p);
              hi = lo = 0;
            }
          }
        }
        y = csub(acc + mont_fold(hi, lo, pr.p, s.pinv[o]), pr.p);
        if (!s.is_one) {
          // whi < 2^63: w mod q_j = whi * 2^64 + wlo in [0, 2q_j) from one
          // Shoup product and a reduction of wlo (conditional subtractions
          // when wlo < 8 q_j), where a 128-bit Barrett takes three times the
          // multiplies.
          const uint64_t lo_red = s.wbig ? csub(csub(csub(wlo, 2 * pr.p2), pr.p2), pr.p)
                                         : csub(mul_shoup_lazy(wlo, 1, s.one_shoup[o], pr.p), pr.p);
          const uint64_t wj = csub(mul_shoup_lazy(whi, s.r64[o], s.r64_shoup[o], pr.p), pr.p) + lo_red;
          y = csub(csub(y + (w_sign ? pr.p2 - wj : wj), pr.p2), pr.p);
        }
      } else {
        uint64_t lo = 0, hi = 0;
        if (!s.is_one) {
          const uint64_t wj = reduce128_lazy(whi, wlo, pr);
          lo = w_sign ? pr.p2 - wj : wj;
        }
        mac128(hi, lo, v_low, s.gamma_neg[o]);
        mac128(hi, lo, v_top, s.gamma_neg_hi[o]);
#pragma unroll
        for (int k = 0; k < MAXF; k++) {
          if (k < (int)F) {
            mac128(hi, lo, r[k], s.omega[o][k]);
            if ((k % 14) == 13) {  // keep the exact sum below 2^128
              lo = reduce128(hi, lo, pr);
              hi = 0;
            }
          }
        }
        y = reduce128(hi, lo, pr);
      }
      if constexpr (TOP > 0) {
        if (fwd_here || dig_here)
          rns_stage_buffer<(MAXF > MAXT ? MAXF : MAXT) * 128>()[(o * (1 << TOP) + t) * G + gi] = y;
        else dst[(uint64_t)o << logn] = y;
      } else {
        dst[(uint64_t)o << logn] = y;
      }
    }
  }
  if constexpr (TOP > 0) {
    if (fwd_here || dig_here) {
      __syncthreads();
      const uint64_t* staged = rns_stage_buffer<(MAXF > MAXT ? MAXF : MAXT) * 128>();
      if (fwd_here) {
        for (uint32_t item = threadIdx.x; item < s.out_len * G; item += 128) {
          const uint32_t o = item / G, g2 = item % G;
          uint64_t x[1 << TOP];
#pragma unroll
          for (int u = 0; u < (1 << TOP); u++) x[u] = staged[(o * (1 << TOP) + u) * G + g2];
          fwd_top_stages<TOP>(x, fe.primes[o]);
          uint64_t* row = out.at(poly, o) + b0 + g2;
#pragma unroll
          for (int u = 0; u < (1 << TOP); u++) row[(uint64_t)u << logb] = x[u];
        }
      } else {
        // Digit d (output limb d) in key limb j: key_switching_key.rs:227-235
        // with rq/mod.rs:518-540, the first forward stages of its transform.
        const uint32_t per_digit = fe.digit_limbs * G;
        const uint32_t pbase = (poly / fe.period) * s.out_len;
        for (uint32_t item = threadIdx.x; item < s.out_len * per_digit; item += 128) {
          const uint32_t d = item / per_digit, rem = item - d * per_digit;
          const uint32_t j = rem / G, g2 = rem % G;
          const DevPrime kp = fe.digit_primes[j];
          uint64_t x[1 << TOP];
#pragma unroll
          for (int u = 0; u < (1 << TOP); u++) {
            const uint64_t v = staged[(d * (1 << TOP) + u) * G + g2];
            x[u] = fe.digit_raw ? v : reduce64_lazy(v, kp);
          }
          fwd_top_stages<TOP>(x, kp);
          uint64_t* row = fe.digits.at(pbase + d, j) + b0 + g2;
#pragma unroll
          for (int u = 0; u < (1 << TOP); u++) row[(uint64_t)u << logb] = x[u];
        }
      }
    }
  }
}

template <int MAXF, int MAXT, bool EXACT = false, int TOP = 0>
void launch_rns_scale(const RnsScalerD& sc, uint32_t logn, PolyRef in, PolyRef out, uint32_t start,
                      uint32_t out_len, uint64_t total, cudaStream_t st, const InverseTop* top = nullptr,
                      const ForwardTop* fwd = nullptr) {
  const RnsScalerHost& h = sc.host;
  const size_t F = h.from_len;
  for (uint32_t first = 0; first < out_len; first += MAXT) {
    const uint32_t n = std::min<uint32_t>(MAXT, out_len - first);
    RnsLaunch<MAXF, MAXT> s;
    memset(&s, 0, sizeof(s));
    s.from_len = (uint32_t)F;
    s.out_len = n;
    s.is_one = h.is_one ? 1 : 0;
    s.shift = (uint32_t)h.theta_garner_shift;
    s.tg_sign = h.theta_gamma_sign ? 1 : 0;
    s.tg_lo = h.theta_gamma_lo;
    s.tg_hi = h.theta_gamma_hi;
    for (size_t k = 0; k < F; k++) {
      s.tgar_lo[k] = h.theta_garner_lo[k];
      s.tgar_hi[k] = h.theta_garner_hi[k];
      s.to_lo[k] = h.theta_omega_lo[k];
      s.to_hi[k] = h.theta_omega_hi[k];
      if (h.theta_omega_sign[k]) s.to_sign |= 1u << k;
    }
    if (EXACT && !sc.mont) throw Error(FHEG_ERR_INTERNAL, "Montgomery scaling needs odd target moduli");
    s.wbig = 1;
    for (uint32_t o = 0; o < n; o++) {
      const size_t j = start + first + o;
      if (EXACT) {
        for (size_t k = 0; k < F; k++) s.omega[o][k] = sc.omega_mont[j * F + k];
        s.gamma_neg[o] = sc.gamma_neg_mont[j];
        s.gamma_neg_hi[o] = sc.gamma_neg_hi_mont[j];
        s.pinv[o] = sc.to_pinv[j];
        const uint64_t q = sc.to_moduli[j];
        s.r64[o] = (uint64_t)(((unsigned __int128)1 << 64) % q);
        s.r64_shoup[o] = shoup(s.r64[o], q);
        s.one_shoup[o] = shoup(1, q);
        if (q <= (1ull << 61)) s.wbig = 0;
      } else {
        for (size_t k = 0; k < F; k++) s.omega[o][k] = h.omega[j * F + k];
        s.gamma_neg[o] = sc.gamma_neg[j];
        s.gamma_neg_hi[o] = sc.gamma_neg_hi[j];
      }
      s.p[o] = sc.to_moduli[j];
      s.bhi[o] = sc.to_bhi[j];
      s.blo[o] = sc.to_blo[j];
    }
    PolyRef o = out;
    o.base += (uint64_t)first << logn;
    FwdEpilogue fe{};
    if (fwd) {
      if (fwd->digit_primes && first > 0) throw Error(FHEG_ERR_INTERNAL, "digit expansion needs one launch");
      fe = FwdEpilogue{fwd->primes + first, fwd->period, fwd->take, fwd->digit_primes, fwd->digit_limbs,
                       fwd->digit_raw, fwd->digits};
    }
    const unsigned threads = 128;
    k_rns_scale<MAXF, MAXT, EXACT, TOP><<<blocks_for(total, threads), threads, 0, st>>>(
        s, logn, in, o, total, top ? top->primes : nullptr, top ? top->mont : 0u, fe);
    after_launch("k_rns_scale");
  }
}

template <int MAXF, int MAXT>
static void launch_rns_scale_top(const RnsScalerD& s, uint32_t logn, PolyRef in, PolyRef out, uint32_t start,
                                 uint32_t out_len, uint64_t total, cudaStream_t st, const InverseTop& top,
                                 const ForwardTop* fwd) {
  switch (top.s1) {
    case 1: launch_rns_scale<MAXF, MAXT, true, 1>(s, logn, in, out, start, out_len, total, st, &top, fwd); break;
    case 2: launch_rns_scale<MAXF, MAXT, true, 2>(s, logn, in, out, start, out_len, total, st, &top, fwd); break;
    case 3: launch_rns_scale<MAXF, MAXT, true, 3>(s, logn, in, out, start, out_len, total, st, &top, fwd); break;
    default: throw Error(FHEG_ERR_INTERNAL, "unsupported strided stage count");
  }
}

bool rns_scale_takes_top(const RnsScalerD& s, uint32_t logn, uint32_t out_len, uint32_t s1) {
  const size_t F = s.host.from_len;
  const bool exact = (F == 6 || F == 13 || F == 3 || F == 7) ? out_len <= 8 : (F == 12 || F == 25) && out_len <= 16;
  return exact && s.mont && s1 >= 1 && s1 <= 3 && logn >= 7;
}

void rns_scale(const RnsScalerD& s, uint32_t logn, PolyRef in, PolyRef out, uint32_t start, uint32_t out_len,
               uint64_t polys, cudaStream_t st, const InverseTop* top, const ForwardTop* fwd) {
  const uint64_t total = polys << logn;
  if (total == 0 || out_len == 0) return;
  const size_t F = s.host.from_len;
  if (fwd && (!top || fwd->s1 != top->s1))
    throw Error(FHEG_ERR_INTERNAL, "forward strided stages need the same count of inverse ones");
  if (top) {
    if (!rns_scale_takes_top(s, logn, out_len, top->s1))
      throw Error(FHEG_ERR_INTERNAL, "RNS scaling cannot apply these strided stages");
    if (F == 6) launch_rns_scale_top<6, 8>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else if (F == 13) launch_rns_scale_top<13, 8>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else if (F == 3) launch_rns_scale_top<3, 8>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else if (F == 7) launch_rns_scale_top<7, 8>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else if (F == 12) launch_rns_scale_top<12, 16>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else launch_rns_scale_top<25, 16>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    return;
  }
  // Exact source counts of the default multiplications at L = 3, 6, 12
  // (extension from L, scale-down from 2L + 1), odd target moduli.
  if (!s.mont) {
    if (F <= 8) launch_rns_scale<8, 8>(s, logn, in, out, start, out_len, total, st);
    else if (F <= 16 && out_len <= 8) launch_rns_scale<16, 8>(s, logn, in, out, start, out_len, total, st);
    else if (F <= 16) launch_rns_scale<16, 16>(s, logn, in, out, start, out_len, total, st);
    else if (F <= 32) launch_rns_scale<32, 16>(s, logn, in, out, start, out_len, total, st);
    else throw Error(FHEG_ERR_UNSUPPORTED, "RNS scaling from more than 32 moduli is not supported");
    return;
  }
  if (F == 6 && out_len <= 8) launch_rns_scale<6, 8, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 13 && out_len <= 8) launch_rns_scale<13, 8, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 3 && out_len <= 8) launch_rns_scale<3, 8, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 7 && out_len <= 8) launch_rns_scale<7, 8, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 12 && out_len <= 16) launch_rns_scale<12, 16, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 25 && out_len <= 16) launch_rns_scale<25, 16, true>(s, logn, in, out, start, out_len, total, st);
  else if (F <= 8) launch_rns_scale<8, 8>(s, logn, in, out, start, out_len, total, st);
  else if (F <= 16 && out_len <= 8) launch_rns_scale<16, 8>(s, logn, in, out, start, out_len, total, st);
  else if (F <= 16) launch_rns_scale<16, 16>(s, logn, in, out, start, out_len, total, st);
  else if (F <= 32) launch_rns_scale<32, 16>(s, logn, in, out, start, out_len, total, st);
  else throw Error(FHEG_ERR_UNSUPPORTED, "RNS scaling from more than 32 moduli is not supported");
}

RnsScalerD::RnsScalerD(const Context& from, const Context& to, const BigUint& num, const BigUint& den)
    : host(make_rns_scaler(*from.rns, *to.rns, num, den)) {
  const size_t T = host.to_len;
  gamma_neg.resize(T);
  gamma_neg_hi.resize(T);
  to_moduli = to.moduli;
  to_bhi.resize(T);
  to_blo.resize(T);
  for (size_t j = 0; j < T; j++) {
    gamma_neg[j] = (to.moduli[j] - host.gamma[j]) % to.moduli[j];
    gamma_neg_hi[j] = mulmod(gamma_neg[j], (1ull << 62) % to.moduli[j], to.moduli[j]);
    barrett128(to.moduli[j], &to_bhi[j], &to_blo[j]);
  }
  mont = true;
  for (size_t j = 0; j < T; j++) mont = mont && (to.moduli[j] & 1);
  if (mont) {
    const size_t F = host.from_len;
    omega_mont.resize(T * F);
    gamma_neg_mont.resize(T);
    gamma_neg_hi_mont.resize(T);
    to_pinv.resize(T);
    for (size_t j = 0; j < T; j++) {
      const uint64_t q = to.moduli[j];
      const uint64_t r = (uint64_t)(((unsigned __int128)1 << 64) % q);
      for (size_t k = 0; k < F; k++) omega_mont[j * F + k] = mulmod(host.omega[j * F + k], r, q);
      gamma_neg_mont[j] = mulmod(gamma_neg[j], r, q);
      gamma_neg_hi_mont[j] = mulmod(gamma_neg_hi[j], r, q);
      uint64_t inv = q;  // q^-1 mod 2^64 by Newton's iteration
      for (int it = 0; it < 6; it++) inv *= 2 - q * inv;
      to_pinv[j] = 0 - inv;
    }
  }
}

Scaler::Scaler(std::shared_ptr<Context> f, std::shared_ptr<Context> t, const BigUint& n, const BigUint& d)
    : from(std::move(f)), to(std::move(t)), num(n), den(d) {
  if (from->degree != to->degree) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Incompatible degrees");
  rns.reset(new RnsScalerD(*from, *to, num, den));
  number_common_moduli = 0;
  if (rns->host.is_one) {  // rq/scaler.rs:32-40
    while (number_common_moduli < from->L() && number_common_moduli < to->L() &&
           from->moduli[number_common_moduli] == to->moduli[number_common_moduli])
      number_common_moduli++;
  }
}

__global__ void k_copy_limbs(PolyRef in, PolyRef out, uint32_t limbs, uint32_t logn, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  const uint32_t limb = job % limbs;
  const uint32_t poly = job / limbs;
  out.at(poly, limb)[i] = in.at(poly, limb)[i];
}

void scaler_scale(const Scaler& s, bool ntt, PolyRef in, PolyRef out, uint64_t polys, uint64_t* scratch,
                  cudaStream_t st) {
  if (polys == 0) return;
  const uint32_t logn = s.from->logn;
  const size_t ncm = s.number_common_moduli;
  const size_t Lt = s.to->L();
  if (ncm > 0) {  // rq/scaler.rs:60-64
    uint64_t total = polys * ncm << logn;
    k_copy_limbs<<<blocks_for(total, 256), 256, 0, st>>>(in, out, (uint32_t)ncm, logn, total);
    after_launch("k_copy_limbs");
  }
  if (ncm >= Lt) return;
  PolyRef src = in;
  if (ntt) {  // rq/scaler.rs:67-81: backward NTT of a copy
    PolyRef tmp = plain_ref(scratch, s.from->L(), logn);
    ntt_backward(*s.from, in, tmp, polys, st);
    src = tmp;
  }
  // Output limbs ncm.. of `out`.
  PolyRef dst = out;
  dst.base = out.base + ((uint64_t)ncm << logn);
  rns_scale(*s.rns, logn, src, dst, (uint32_t)ncm, (uint32_t)(Lt - ncm), polys, st);
  if (ntt) {  // rq/scaler.rs:96-114: forward NTT of the new limbs.
    // The target context restricted to limbs ncm.. : same tables, offset primes.
    NttGeom g{s.to->primes_dev() + ncm, (uint32_t)(Lt - ncm), 0};
    ntt_forward_any<true>(logn, g, polys, SrcPoly{dst}, DstPoly{dst}, st);
  }
}

}  // namespace fheg
