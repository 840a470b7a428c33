// workload.cpp - host generator of bank transaction streams (format in include/csmv.h).
//
// The reference draws addresses inside the kernel from a per-thread LCG (RAND_R_FNC,
// bank/csmv_sh/API.cuh:37-53) whose state advances on every retry, so a retried transaction
// touches different accounts and no two runs execute the same transactions. Here a stream is
// an explicit, seeded list: transaction i's draws come from a counter hash of (seed, i, draw),
// a retry re-executes the same transaction, and the CPU replay and baselines consume exactly
// the stream the GPU ran.
#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"

namespace {

inline uint64_t mix64(uint64_t x) {  // splitmix64 finalizer
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
inline uint64_t draw64(uint64_t seed, uint64_t a, uint64_t b) {
  return mix64(mix64(seed + 0xD6E8FEB86659FD93ull * a) ^ b);
}
inline uint32_t draw32(uint64_t seed, uint64_t a, uint64_t b) {
  return static_cast<uint32_t>(draw64(seed, a, b) >> 32);
}
inline uint32_t scale(uint32_t r, uint32_t n) {  // multiply-shift into [0, n)
  return static_cast<uint32_t>((static_cast<uint64_t>(r) * n) >> 32);
}

// Zipf(theta) over ranks 1..n by rejection-inversion (W. Hormann and G. Derflinger,
// "Rejection-inversion to generate variates from monotone discrete distributions",
// ACM TOMACS 6(3):169-184, 1996). H is the integral of h(x) = x^-theta written as
// log(x) * expm1((1-theta) log x) / ((1-theta) log x) and Hinv its inverse through log1p, so
// both stay accurate as theta approaches 1; the helpers log1p(x)/x and expm1(x)/x fall back to
// their Taylor series near 0. This numerically stable form is the one of the widely published
// Apache Commons Math sampler (RejectionInversionZipfSampler), restated here.
class Zipf {
 public:
  Zipf(double theta, uint32_t n) : s_(theta), n_(n) {
    hx1_ = H(1.5) - 1.0;
    hn_ = H(n_ + 0.5);
    shift_ = 2.0 - Hinv(H(2.5) - h(2.0));
  }
  uint32_t rank(uint64_t seed, uint64_t i, uint64_t c) const {
    for (uint32_t it = 0; it < 256; ++it) {
      const double u01 = static_cast<double>(draw64(seed, i, 0x10000ull + (c << 8) + it) >> 11) * 0x1p-53;
      const double u = hn_ + u01 * (hx1_ - hn_);
      const double x = Hinv(u);
      double k = std::floor(x + 0.5);
      if (k < 1.0) k = 1.0;
      if (k > n_) k = n_;
      if (k - x <= shift_ || u >= H(k + 0.5) - h(k)) return static_cast<uint32_t>(k);
    }
    return 1;
  }

 private:
  static double log1p_over(double x) {
    return std::fabs(x) > 1e-8 ? std::log1p(x) / x : 1.0 - x * (0.5 - x * (1.0 / 3.0 - 0.25 * x));
  }
  static double expm1_over(double x) {
    return std::fabs(x) > 1e-8 ? std::expm1(x) / x
                               : 1.0 + x * 0.5 * (1.0 + x * (1.0 / 3.0) * (1.0 + 0.25 * x));
  }
  double H(double x) const {
    const double lx = std::log(x);
    return expm1_over((1.0 - s_) * lx) * lx;
  }
  double h(double x) const { return std::exp(-s_ * std::log(x)); }
  double Hinv(double x) const {
    double t = x * (1.0 - s_);
    if (t < -1.0) t = -1.0;
    return std::exp(log1p_over(t) * x);
  }
  double s_, n_, hx1_, hn_, shift_;
};

bool round_is_readonly(const csmv_bank_workload& w, uint32_t round) {
  return scale(draw32(w.seed, (1ull << 40) + round, 0), 100) < w.pr_read_pct;
}

struct AccountDraw {
  const csmv_bank_workload& w;
  Zipf zipf;
  uint32_t hot_n;
  explicit AccountDraw(const csmv_bank_workload& wl)
      : w(wl), zipf(wl.dist == CSMV_DIST_ZIPF ? wl.zipf_theta : 1.0, wl.n_accounts) {
    double hn = wl.hot_frac * static_cast<double>(wl.n_accounts);
    hot_n = hn < 1.0 ? 1u : static_cast<uint32_t>(hn);
  }
  uint32_t operator()(uint64_t i, uint64_t c) const {
    const uint32_t n = w.n_accounts;
    switch (w.dist) {
      case CSMV_DIST_ZIPF:
        return zipf.rank(w.seed, i, c) - 1u;
      case CSMV_DIST_HOTSPOT: {
        const uint64_t epoch = w.shift_every ? i / w.shift_every : 0;
        const uint32_t base = scale(draw32(w.seed, (2ull << 40) + epoch, 0), n);
        const uint32_t r1 = draw32(w.seed, i, 0x100ull + 2 * c);
        const uint32_t r2 = draw32(w.seed, i, 0x101ull + 2 * c);
        if (static_cast<double>(r1) < w.hot_prob * 4294967296.0)
          return static_cast<uint32_t>((static_cast<uint64_t>(base) + scale(r2, hot_n)) % n);
        return scale(r2, n);
      }
      default:
        return scale(draw32(w.seed, i, 0x100ull + 2 * c), n);
    }
  }
};

csmv_status check_workload(const csmv_bank_workload* w) {
  if (!w || w->n_txn == 0 || w->n_txn % 32 || w->n_accounts < 2 || w->up_reads < 2 ||
      w->up_reads > 32 || w->up_reads > w->n_accounts /* a transfer's accounts are distinct */ ||
      w->ro_reads < 1 || w->ro_reads > 32 || w->amt_lo < 1 ||
      w->amt_hi < w->amt_lo || w->amt_hi > 4095 || w->pr_read_pct > 100 ||
      (w->kind != CSMV_KIND_TRANSFER && w->kind != CSMV_KIND_TRANSFER_ALWAYS) || w->dist > 2 ||
      (w->dist == CSMV_DIST_HOTSPOT && !(w->hot_frac > 0.0 && w->hot_frac <= 1.0))) {
    csmv::set_error("invalid bank workload");
    return CSMV_ERR_INVALID_ARG;
  }
  return CSMV_OK;
}

}  // namespace

extern "C" csmv_status csmv_bank_stream_size(const csmv_bank_workload* w, uint64_t* n_addr) {
  csmv_status st = check_workload(w);
  if (st != CSMV_OK) return st;
  if (!n_addr) return CSMV_ERR_INVALID_ARG;
  uint64_t total = 0;
  for (uint32_t r = 0; r < w->n_txn / 32; ++r)
    total += 32ull * (round_is_readonly(*w, r) ? w->ro_reads : w->up_reads);
  *n_addr = total;
  return CSMV_OK;
}

extern "C" csmv_status csmv_bank_generate(const csmv_bank_workload* w, uint32_t* op, uint32_t* off,
                                          uint32_t* addr) {
  csmv_status st = check_workload(w);
  if (st != CSMV_OK) return st;
  if (!op || !off || !addr) return CSMV_ERR_INVALID_ARG;
  const AccountDraw draw(*w);
  uint64_t pos = 0;
  for (uint32_t r = 0; r < w->n_txn / 32; ++r) {
    const bool ro = round_is_readonly(*w, r);
    for (uint32_t lane = 0; lane < 32; ++lane) {
      const uint64_t i = static_cast<uint64_t>(r) * 32 + lane;
      off[i] = static_cast<uint32_t>(pos);
      if (ro) {
        op[i] = CSMV_MAKE_OP(CSMV_KIND_READONLY, w->ro_reads, 1, 1);
        for (uint32_t k = 0; k < w->ro_reads; ++k) addr[pos++] = draw(i, k * 64ull);
        continue;
      }
      const uint32_t amt0 = w->amt_lo + scale(draw32(w->seed, i, 1), w->amt_hi - w->amt_lo + 1);
      op[i] = CSMV_MAKE_OP(w->kind, w->up_reads, amt0, w->amt_hi);
      uint32_t* mine = addr + pos;
      for (uint32_t k = 0; k < w->up_reads; ++k) {
        auto used = [&](uint32_t a) {
          for (uint32_t j = 0; j < k; ++j)
            if (mine[j] == a) return true;
          return false;
        };
        uint32_t a = 0;
        bool ok = false;
        for (uint32_t att = 0; att < 64 && !ok; ++att) {
          a = draw(i, k * 64ull + att);
          ok = !used(a);
        }
        while (!ok) {  // only reachable with a handful of accounts
          a = (a + 1) % w->n_accounts;
          ok = !used(a);
        }
        mine[k] = a;
      }
      pos += w->up_reads;
    }
  }
  return CSMV_OK;
}

// ---------------------------------------------------------------------------------------------
// cache requests
// ---------------------------------------------------------------------------------------------
namespace {
csmv_status check_memcd_workload(const csmv_memcd_workload* w) {
  if (!w || w->n_req == 0 || w->n_req % 32 || w->n_keys < 1 || w->get_pct > 100 ||
      (w->dist != CSMV_DIST_UNIFORM && w->dist != CSMV_DIST_ZIPF) ||
      (w->dist == CSMV_DIST_ZIPF && !(w->zipf_theta > 0.0))) {
    csmv::set_error("invalid memcd workload");
    return CSMV_ERR_INVALID_ARG;
  }
  return CSMV_OK;
}
}  // namespace

extern "C" csmv_status csmv_memcd_generate(const csmv_memcd_workload* w, uint32_t* kind,
                                           uint32_t* key, uint32_t* val) {
  csmv_status st = check_memcd_workload(w);
  if (st != CSMV_OK) return st;
  if (!kind || !key || !val) return CSMV_ERR_INVALID_ARG;
  const Zipf zipf(w->dist == CSMV_DIST_ZIPF ? w->zipf_theta : 1.0, w->n_keys);
  for (uint32_t r = 0; r < w->n_req / 32; ++r) {
    const bool get = scale(draw32(w->seed, (3ull << 40) + r, 0), 100) < w->get_pct;
    for (uint32_t lane = 0; lane < 32; ++lane) {
      const uint64_t i = static_cast<uint64_t>(r) * 32 + lane;
      kind[i] = get ? CSMV_MEMCD_GET : CSMV_MEMCD_SET;
      const uint32_t id = w->dist == CSMV_DIST_ZIPF ? zipf.rank(w->seed, i, 0) - 1u
                                                    : scale(draw32(w->seed, i, 0x100ull), w->n_keys);
      key[4 * i] = id;
      for (uint32_t j = 1; j < 4; ++j) key[4 * i + j] = static_cast<uint32_t>(mix64(id * 4ull + j) >> 32);
      for (uint32_t j = 0; j < 8; ++j) val[8 * i + j] = get ? 0u : draw32(w->seed, i, 0x200ull + j);
    }
  }
  return CSMV_OK;
}
