// csmv_memcd - cache driver with the reference's command line (memcachedGPU/memcdSH.cu:490-529):
//
//   csmv_memcd <seed> <nbSets> <nbWays> <serverThreads> <clientBlocks> <clientThreads>
//              <nbTXsPerThread> <prRead%> <duration_s> <verbose>
//
// Each iteration draws clientBlocks*clientThreads*nbTXsPerThread requests, keys uniform over
// nbSets*nbWays*2 key ids as in the reference (memcdSH.cu:536,624-634), and runs them as one
// batch; the LRU tick starts at 1 and advances after every batch (memcdSH.cu:573,648). The loop
// ends once the summed kernel time reaches duration_s (memcdSH.cu:622). Output: the reference's
// line - abort %, committed requests/s, DataAge/RecordAge/ReadWrite/PreValidation abort % - then
// its 17 clock64 phase-time fields as 0 (not instrumented here), the iteration count, and extra
// fields: write-lock abort %, kernel ms, GETs, SETs, GET hits, p50 and p99 batch latency (ms).
//
// Differences, all deliberate: keys are 16 bytes and values 32 bytes (4 and 8 words, the
// reference's KEY_SIZE/VAL_SIZE words all hold the key id); rounds of 32 requests are all GETs or
// all SETs with probability prRead% per round (the reference draws it per warp per transaction);
// clientThreads/32 client warps per CTA share their CTA's commit-server warp, so serverThreads is
// accepted but unused. CSMV_MEMCD_MAX_ITERS bounds the iteration count (default unbounded).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "csmv.h"

static const char* kHelp =
    "argument order:                     \n"
    "  1) rng seed                       \n"
    "  2) nb sets in cache               \n"
    "  3) nb ways per set                \n"
    "  4) server config - nb threads     \n"
    "  5) client config - nb blocks      \n"
    "  6) client config - nb threads     \n"
    "  7) nb TXs per thread              \n"
    "  8) prob read TX kernel            \n"
    "  9) run duration                   \n"
    " 10) verbose                        \n";

int main(int argc, char** argv) {
  if (argc != 11) {
    std::printf("%s\n", kHelp);
    return 0;
  }
  const uint64_t seed = std::strtoull(argv[1], nullptr, 10);
  const uint32_t n_sets = (uint32_t)std::atol(argv[2]);
  const uint32_t n_ways = (uint32_t)std::atol(argv[3]);
  const uint32_t blocks = (uint32_t)std::atol(argv[5]);
  const uint32_t threads = (uint32_t)std::atol(argv[6]);
  const uint32_t per_thread = (uint32_t)std::atol(argv[7]);
  const uint32_t pr_read = (uint32_t)std::atol(argv[8]);
  const double duration_s = std::atof(argv[9]);
  const int verbose = std::atoi(argv[10]);
  const char* mi = std::getenv("CSMV_MEMCD_MAX_ITERS");
  const long max_iters = mi && *mi ? std::atol(mi) : -1;
  if (n_ways != CSMV_MEMCD_WAYS) {
    std::fprintf(stderr, "nbWays must be %d\n", CSMV_MEMCD_WAYS);
    return 1;
  }
  if (threads < 32 || threads % 32 || blocks < 1 || per_thread < 1 || pr_read > 100) {
    std::fprintf(stderr, "clientThreads must be a multiple of 32; blocks, TXs >= 1\n");
    return 1;
  }
  const uint64_t n64 = (uint64_t)blocks * threads * per_thread;
  if (n64 > (1ull << 26)) {
    std::fprintf(stderr, "batch too large\n");
    return 1;
  }
  const uint32_t n = (uint32_t)n64;

  csmv_memcd_config cfg;
  csmv_memcd_config_default(&cfg);
  cfg.n_sets = n_sets;
  cfg.client_warps = threads / 32;
  cfg.ctas = blocks;
  cfg.max_req = n;
  cfg.log_commits = 0;
  csmv_memcd_t* h = nullptr;
  csmv_status st = csmv_memcd_create(&cfg, &h);
  if (st == CSMV_OK) st = csmv_memcd_clear(h);
  if (st != CSMV_OK) {
    std::fprintf(stderr, "csmv_memcd_create: %s: %s\n", csmv_status_str(st), csmv_last_error());
    return 1;
  }
  std::vector<uint32_t> kind(n), key(4ull * n), val(8ull * n), found(n), out(8ull * n);
  csmv_memcd_workload w;
  std::memset(&w, 0, sizeof(w));
  w.n_keys = n_sets * n_ways * 2;
  w.n_req = n;
  w.get_pct = pr_read;
  w.dist = CSMV_DIST_UNIFORM;

  double kernel_ms = 0.0;
  uint64_t commits = 0, aborts = 0, a_age = 0, a_rw = 0, a_pv = 0, a_ww = 0, gets = 0, sets = 0,
           hits = 0;
  std::vector<double> lat;
  long iters = 0;
  while (kernel_ms < duration_s * 1000.0 && (max_iters < 0 || iters < max_iters)) {
    w.seed = seed + (uint64_t)iters;  // regenerate keys every batch (memcdSH.cu:624-634)
    if ((st = csmv_memcd_generate(&w, kind.data(), key.data(), val.data())) != CSMV_OK) break;
    csmv_memcd_batch b{n, (uint32_t)(iters + 1), kind.data(), key.data(), val.data(),
                       found.data(), out.data()};
    csmv_stats s;
    if ((st = csmv_memcd_run(h, &b, &s)) != CSMV_OK) break;
    kernel_ms += s.kernel_ms;
    lat.push_back(s.total_ms);
    commits += s.commits_update + s.commits_readonly;
    a_age += s.aborts_data_age;
    a_rw += s.aborts_read_write;
    a_pv += s.aborts_prevalid;
    a_ww += s.aborts_write_write;
    gets += s.commits_readonly;
    sets += s.commits_update;
    for (uint32_t i = 0; i < n; i++) hits += found[i];
    iters++;
  }
  csmv_memcd_destroy(h);
  if (st != CSMV_OK) {
    std::fprintf(stderr, "csmv_memcd: %s: %s\n", csmv_status_str(st), csmv_last_error());
    return 1;
  }
  aborts = a_age + a_rw + a_pv + a_ww;
  const double tot = commits + aborts > 0 ? (double)(commits + aborts) : 1.0;
  const double tput = kernel_ms > 0 ? commits / kernel_ms * 1000.0 : 0.0;
  std::sort(lat.begin(), lat.end());
  auto pct = [&](double q) {
    return lat.empty() ? 0.0 : lat[std::min(lat.size() - 1, (size_t)(q * (lat.size() - 1) + 0.5))];
  };
  if (verbose) {
    std::printf(
        "AbortPercent\t%f %%\nThroughtput\t%f\n\nAbortDataAge\t%f %%\nAbortRecAge\t%f %%\n"
        "AbortReadWrite\t%f %%\nAbortPreVal\t%f %%\nAbortWriteLock\t%f %%\n\nKernelMs\t%f\n"
        "Gets\t\t%llu\nSets\t\t%llu\nHits\t\t%llu\nBatchP50Ms\t%f\nBatchP99Ms\t%f\nTotalIters\t%ld\n",
        aborts / tot * 100.0, tput, a_age / tot * 100.0, 0.0, a_rw / tot * 100.0,
        a_pv / tot * 100.0, a_ww / tot * 100.0, kernel_ms, (unsigned long long)gets,
        (unsigned long long)sets, (unsigned long long)hits, pct(0.5), pct(0.99), iters);
  } else {
    std::printf("%f\t%f\t%f\t%f\t%f\t%f", aborts / tot * 100.0, tput, a_age / tot * 100.0, 0.0,
                a_rw / tot * 100.0, a_pv / tot * 100.0);
    for (int i = 0; i < 17; i++) std::printf("\t%f", 0.0);
    std::printf("\t%ld\t%f\t%f\t%llu\t%llu\t%llu\t%f\t%f\n", iters, a_ww / tot * 100.0, kernel_ms,
                (unsigned long long)gets, (unsigned long long)sets, (unsigned long long)hits,
                pct(0.5), pct(0.99));
  }
  return 0;
}
