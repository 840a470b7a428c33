// csmv_bank - bank driver with the reference's command line (bank/csmv_sh/exe.cu:531-575):
//
//   csmv_bank <nbAccounts> <clientThreads> <clientBlocks> <serverThreads> <prRead%> <roSize>
//             <upSize> <verbose>
//
// and the reference's output: one tab-separated line starting with abort %, throughput
// (committed tx/s, read-only included), then DataAge/RecordAge/ReadWrite/PreValidation abort %
// (exe.cu:499-523); the reference's 17 clock64 phase-time fields follow as 0 (this engine does
// not instrument phases with clock64), then extra fields: kernel ms, commits, rounds, sections.
//
// Differences, all deliberate: runs are count-bounded (CSMV_TX_PER_THREAD transactions per
// client thread, default 256) instead of a 5 s sleep; clientThreads/32 client warps per CTA each
// share their CTA's commit-server warp, so serverThreads is accepted but unused; upSize k means a
// transfer that reads 2k accounts and writes two (the reference writes all 2k).
// Engine options come from the environment: CSMV_VALIDATE (stamp|ring|ring_lane),
// CSMV_BATCH (lane|warp|cta), CSMV_WRITEBACK (client|server), CSMV_PREVALIDATE (0|1),
// CSMV_DEPTH (2|4|8|16), CSMV_SEED. Traces: CSMV_TRACE_IN=<file> runs the stream of a stream
// file (csmv_stream_save) instead of generating one; CSMV_TRACE_OUT=<prefix> writes the run's
// stream to <prefix>.stream and its commit log to <prefix>.log (csmv_log_save), so the same run
// can be replayed and checked on the CPU.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "csmv.h"

static const char* kHelp =
    "argument order:                     \n"
    "  1) nb bank accounts               \n"
    "  2) client config - nb threads     \n"
    "  3) client config - nb blocks      \n"
    "  4) server config - nb threads     \n"
    "  5) prob read TX                   \n"
    "  6) read TX Size                   \n"
    "  7) update TX Size                 \n"
    "  8) verbose                        \n";

static uint32_t env_u32(const char* name, uint32_t dflt) {
  const char* v = std::getenv(name);
  return v && *v ? (uint32_t)std::strtoul(v, nullptr, 10) : dflt;
}

static uint32_t env_choice(const char* name, const char* const* names, uint32_t n, uint32_t dflt) {
  const char* v = std::getenv(name);
  if (!v || !*v) return dflt;
  for (uint32_t i = 0; i < n; i++)
    if (!std::strcmp(v, names[i])) return i;
  std::fprintf(stderr, "%s=%s not understood; using default\n", name, v);
  return dflt;
}

int main(int argc, char** argv) {
  if (argc != 9) {
    std::printf("%s\n", kHelp);
    return 0;
  }
  const uint32_t n_accounts = (uint32_t)std::atoi(argv[1]);
  const uint32_t client_threads = (uint32_t)std::atoi(argv[2]);
  const uint32_t client_blocks = (uint32_t)std::atoi(argv[3]);
  const uint32_t server_threads = (uint32_t)std::atoi(argv[4]);
  const uint32_t pr_read = (uint32_t)std::atoi(argv[5]);
  const uint32_t ro_size = (uint32_t)std::atoi(argv[6]);
  const uint32_t up_size = (uint32_t)std::atoi(argv[7]);
  const int verbose = std::atoi(argv[8]);
  (void)server_threads;
  if (client_threads < 32 || client_threads % 32 || client_blocks < 1 || up_size < 1) {
    std::fprintf(stderr, "clientThreads must be a multiple of 32, clientBlocks and upSize >= 1\n");
    return 1;
  }

  csmv_bank_config cfg;
  csmv_bank_config_default(&cfg);
  static const char* kValidate[] = {"stamp", "ring", "ring_lane"};
  static const char* kBatch[] = {"lane", "warp", "cta"};
  static const char* kWb[] = {"client", "server"};
  cfg.n_accounts = n_accounts;
  cfg.init_value = 100;  // bank/csmv_sh/exe.cu:373-376
  cfg.client_warps = client_threads / 32;
  cfg.ctas = client_blocks;
  cfg.validate = env_choice("CSMV_VALIDATE", kValidate, 3, CSMV_VALIDATE_STAMP);
  cfg.batch = env_choice("CSMV_BATCH", kBatch, 3, CSMV_BATCH_CTA);
  cfg.writeback = env_choice("CSMV_WRITEBACK", kWb, 2,
                             cfg.batch == CSMV_BATCH_LANE ? CSMV_WRITEBACK_SERVER : CSMV_WRITEBACK_CLIENT);
  cfg.prevalidate = env_u32("CSMV_PREVALIDATE", 1);
  cfg.version_depth = env_u32("CSMV_DEPTH", 4);
  const uint32_t per_thread = env_u32("CSMV_TX_PER_THREAD", 256);
  const uint64_t n_txn64 = (uint64_t)client_threads * client_blocks * per_thread;
  if (n_txn64 > 0xFFFFFFE0ull) {
    std::fprintf(stderr, "too many transactions\n");
    return 1;
  }
  const uint32_t n_txn = (uint32_t)n_txn64;
  cfg.max_txn = n_txn;
  cfg.log_commits = 0;

  csmv_bank_workload w;
  std::memset(&w, 0, sizeof(w));
  w.seed = env_u32("CSMV_SEED", 1);
  w.n_accounts = n_accounts;
  w.n_txn = n_txn;
  w.pr_read_pct = pr_read;
  w.ro_reads = ro_size < 1 ? 1 : (ro_size > 32 ? 32 : ro_size);
  w.up_reads = 2 * up_size > 8 ? 8 : 2 * up_size;
  w.kind = CSMV_KIND_TRANSFER_ALWAYS;  // the reference's unconditional -1/+1 transfer
  w.amt_lo = w.amt_hi = 1;
  w.dist = CSMV_DIST_UNIFORM;
  uint64_t n_addr = 0;
  csmv_status st = csmv_bank_stream_size(&w, &n_addr);
  if (st != CSMV_OK) {
    std::fprintf(stderr, "workload: %s\n", csmv_last_error());
    return 1;
  }
  std::vector<uint32_t> op(n_txn), off(n_txn), addr(n_addr);
  csmv_bank_generate(&w, op.data(), off.data(), addr.data());
  uint32_t run_txn = n_txn;
  if (const char* in = std::getenv("CSMV_TRACE_IN")) {
    uint32_t t = 0;
    uint64_t a = 0;
    if ((st = csmv_stream_info(in, &t, &a)) != CSMV_OK) {
      std::fprintf(stderr, "CSMV_TRACE_IN: %s\n", csmv_last_error());
      return 1;
    }
    op.assign(t, 0);
    off.assign(t, 0);
    addr.assign(a, 0);
    if ((st = csmv_stream_load(in, op.data(), off.data(), addr.data(), t, a)) != CSMV_OK) {
      std::fprintf(stderr, "CSMV_TRACE_IN: %s\n", csmv_last_error());
      return 1;
    }
    run_txn = t;
    n_addr = a;
    cfg.max_txn = t > 0 ? t : 32;
  }
  const char* trace_out = std::getenv("CSMV_TRACE_OUT");
  if (trace_out) cfg.log_commits = 1;

  csmv_bank_t* h = nullptr;
  if ((st = csmv_bank_create(&cfg, &h)) != CSMV_OK) {
    std::fprintf(stderr, "csmv_bank_create: %s: %s\n", csmv_status_str(st), csmv_last_error());
    return 1;
  }
  if ((st = csmv_bank_load(h, nullptr)) != CSMV_OK) {
    std::fprintf(stderr, "csmv_bank_load: %s\n", csmv_last_error());
    return 1;
  }
  csmv_bank_stream s{run_txn, op.data(), off.data(), addr.data(), n_addr};
  if (trace_out) {
    const std::string path = std::string(trace_out) + ".stream";
    if ((st = csmv_stream_save(path.c_str(), &s)) != CSMV_OK) {
      std::fprintf(stderr, "CSMV_TRACE_OUT: %s\n", csmv_last_error());
      csmv_bank_destroy(h);
      return 1;
    }
  }
  csmv_stats stats;
  st = csmv_bank_run(h, &s, &stats);
  if (st != CSMV_OK) {
    std::fprintf(stderr, "csmv_bank_run: %s: %s\n", csmv_status_str(st), csmv_last_error());
    csmv_bank_destroy(h);
    return 1;
  }
  if (trace_out) {  // timestamps 1..final_ts of this (first) run, holes included
    std::vector<uint32_t> log_txn(stats.final_ts > 0 ? stats.final_ts : 1), outcome(run_txn);
    std::vector<int32_t> result(run_txn);
    const std::string path = std::string(trace_out) + ".log";
    if ((st = csmv_bank_read_log(h, log_txn.data(), stats.final_ts, outcome.data(), result.data(),
                                 run_txn)) != CSMV_OK ||
        (st = csmv_log_save(path.c_str(), 0, log_txn.data(), stats.final_ts, outcome.data(),
                            result.data(), run_txn)) != CSMV_OK) {
      std::fprintf(stderr, "CSMV_TRACE_OUT: %s\n", csmv_last_error());
      csmv_bank_destroy(h);
      return 1;
    }
  }
  // TXEnd's invariant (bank/csmv_sh/API.cu:339-350)
  std::vector<int32_t> vals(n_accounts);
  csmv_bank_read_values(h, vals.data());
  long long total = 0;
  for (int32_t v : vals) total += v;
  if (total != 100ll * n_accounts) std::printf("Consistency fail: Total %lld\n", total);
  csmv_bank_destroy(h);

  const double commits = (double)(stats.commits_update + stats.commits_readonly + stats.commits_nowrite);
  const double aborts = (double)(stats.aborts_data_age + stats.aborts_record_age +
                                 stats.aborts_read_write + stats.aborts_prevalid);
  const double tot = commits + aborts > 0 ? commits + aborts : 1.0;
  const double tput = stats.kernel_ms > 0 ? commits / stats.kernel_ms * 1000.0 : 0.0;
  if (verbose) {
    std::printf(
        "AbortPercent\t%f %%\nThroughtput\t%f\n\nAbortDataAge\t%f %%\nAbortRecAge\t%f %%\n"
        "AbortReadWrite\t%f %%\nAbortPreVal\t%f %%\n\nKernelMs\t%f\nCommits\t\t%.0f\n"
        "Rounds\t\t%llu\nSections\t%llu\nTotalUpdates\t%llu\nTotalReads\t%llu\n",
        aborts / tot * 100.0, tput, stats.aborts_data_age / tot * 100.0,
        stats.aborts_record_age / tot * 100.0, stats.aborts_read_write / tot * 100.0,
        stats.aborts_prevalid / tot * 100.0, stats.kernel_ms, commits,
        (unsigned long long)stats.rounds, (unsigned long long)stats.sections,
        (unsigned long long)stats.commits_update, (unsigned long long)stats.commits_readonly);
  } else {
    std::printf("%f\t%f\t%f\t%f\t%f\t%f", aborts / tot * 100.0, tput,
                stats.aborts_data_age / tot * 100.0, stats.aborts_record_age / tot * 100.0,
                stats.aborts_read_write / tot * 100.0, stats.aborts_prevalid / tot * 100.0);
    for (int i = 0; i < 17; i++) std::printf("\t%f", 0.0);
    std::printf("\t%f\t%.0f\t%llu\t%llu\n", stats.kernel_ms, commits,
                (unsigned long long)stats.rounds, (unsigned long long)stats.sections);
  }
  return 0;
}
