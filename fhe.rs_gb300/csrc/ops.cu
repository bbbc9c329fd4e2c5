// Ring-level operations: contexts, NTTs, element-wise ops, substitution and
// modulus switch-down (fhe-math `rq`, `ntt`); RNS scaling is in scale.cu.

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
