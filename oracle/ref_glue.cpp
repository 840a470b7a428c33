/*
 * ref_glue.cpp - exposes the reference's own device functions, compiled for the host, to the
 * oracle tests. TEST INFRASTRUCTURE ONLY: built by oracle/ref_build.sh into oracle/_ref/ from the
 * reference sources where they lie (nothing is copied), and used only to pin the oracle's
 * restatements (tests/test_ref_pin.py) and to generate tests/golden/ fixtures.
 *
 * Compiled functions (paths relative to the reference project root):
 *   bank/csmv_sh/API.cu                                   TXRead, TXReadOnly, TXWriteBack,
 *                                                         TXValidate, TXAddToRecord, TXWrite
 *   csmv_optimizations/batchedAtrInsert/csmv_sh/API.cu    TXValidate, TXPreValidation
 *   RAND_R_FNC (bank/csmv_sh/API.cuh:37-53)
 */
#include "ref_shim.h"

#include <barrier>
#include <thread>

thread_local ref_dim3 threadIdx;

/* ---- 32-thread warp emulator: every collective is a barrier-separated exchange ---- */
static thread_local unsigned tl_lane;
static std::barrier<>* g_bar;
static int g_vals[32];

unsigned ref_emu_lane(void) { return tl_lane; }
unsigned ref_emu_ballot(int pred) {
  g_vals[tl_lane] = pred != 0;
  g_bar->arrive_and_wait();
  unsigned b = 0;
  for (int i = 0; i < 32; i++)
    if (g_vals[i]) b |= 1u << i;
  g_bar->arrive_and_wait();
  return b;
}
int ref_emu_shfl(int v, int src) {
  g_vals[tl_lane] = v;
  g_bar->arrive_and_wait();
  int r = g_vals[src & 31];
  g_bar->arrive_and_wait();
  return r;
}
void ref_emu_sync(void) { g_bar->arrive_and_wait(); }

template <class F>
static void run_warp(F f) {
  std::barrier<> bar(32);
  g_bar = &bar;
  std::thread th[32];
  for (unsigned l = 0; l < 32; l++)
    th[l] = std::thread([&f, l] {
      tl_lane = l;
      threadIdx = ref_dim3{l, 0, 0};
      f(l);
    });
  for (auto& t : th) t.join();
  g_bar = nullptr;
}

/* ---- reference sources, each in its own namespace ---- */
namespace ref_sh {
#include "bank/csmv_sh/API.cu"
}
#undef STM_API_H
#undef MaxWriteSetSize
#undef MaxReadSetSize
#undef TXRecordSize
#undef MaxVersions
#undef bufDec
#undef bufInc
#undef advance_pointer
#undef decrease_pointer
#undef CUDA_CHECK_ERROR
#undef RAND_R_FNC
#undef max
namespace ref_bt {
#include "csmv_optimizations/batchedAtrInsert/csmv_sh/API.cu"
}

struct orc_record_c {
  uint32_t txn, n_writes, ws[4];
};

extern "C" {

uint64_t ref_rand_r(uint64_t* state) {
  uint64_t s = *state;
  uint64_t r = RAND_R_FNC(s);
  *state = s;
  return r;
}

int ref_sh_maxversions(void) { return 10; }
int ref_sh_ring_size(void) { return 1600; }
int ref_bt_ring_size(void) { return 2000; }

/* TXRead (readonly = 0) or TXReadOnly (readonly = 1) on one item; returns 1 on abort */
int ref_sh_read(uint16_t head, uint16_t tail, const uint32_t* version, const int32_t* value,
                uint32_t ts, int readonly, int32_t* out) {
  static ref_sh::VertionedDataItem item;
  static ref_sh::readSet rs[1];
  static ref_sh::writeSet ws[1];
  item.head_ptr = head;
  item.tail_ptr = tail;
  for (int i = 0; i < 10; i++) {
    item.version[i] = version[i];
    item.value[i] = value[i];
  }
  ref_sh::local_metadata md;
  memset(&md, 0, sizeof(md));
  md.timestamp = (int)ts;
  rs[0].size = 0;
  ws[0].size = 0;
  int v = readonly ? ref_sh::TXReadOnly(&item, 0, &md, rs, 0) : ref_sh::TXRead(&item, 0, &md, rs, ws, 0);
  *out = v;
  return md.isAborted ? 1 : 0;
}

/* TXWriteBack of one (item, value) at ts; the item state is updated in place */
void ref_sh_writeback(uint16_t* head, uint16_t* tail, uint32_t* version, int32_t* value,
                      uint32_t ts, int32_t v) {
  static ref_sh::VertionedDataItem item;
  item.head_ptr = *head;
  item.tail_ptr = *tail;
  for (int i = 0; i < 10; i++) {
    item.version[i] = version[i];
    item.value[i] = value[i];
  }
  ref_sh::writeSet ws;
  ws.size = 1;
  ws.addrs[0] = 0;
  ws.value[0] = v;
  ref_sh::globalClock = ts - 1; /* TXWriteBack spins until it may advance the clock to ts */
  ref_sh::TXWriteBack((int)ts, &item, ws);
  *head = item.head_ptr;
  *tail = item.tail_ptr;
  for (int i = 0; i < 10; i++) {
    version[i] = item.version[i];
    value[i] = item.value[i];
  }
}

static void fill_sh_records(ref_sh::TXRecord* r, const orc_record_c* recs) {
  for (int i = 0; i < 1600; i++) {
    r[i].transactionNumber = recs[i].txn;
    r[i].n_writes = (ushort)recs[i].n_writes;
    r[i].writeSet[0] = recs[i].ws[0];
    r[i].writeSet[1] = recs[i].ws[1];
    r[i].recordCommitted = true;
  }
}

/* plain TXValidate; returns 0 valid, 1 RecordAge, 2 ReadWrite */
int ref_sh_validate(const orc_record_c* recs, int hp, int tp, int oldhp, int ts,
                    const uint32_t* rs, int nrs) {
  static ref_sh::TXRecord r[1600];
  static ref_sh::readSet rd;
  static ref_sh::writeSet wr;
  fill_sh_records(r, recs);
  rd.size = (ushort)nrs;
  for (int k = 0; k < nrs; k++) rd.addrs[k] = rs[k];
  wr.size = 0;
  ref_sh::TMmetadata md = {(ushort)tp, (ushort)hp, hp};
  ref_sh::Statistics st;
  memset(&st, 0, sizeof(st));
  static ref_sh::time_rate times[1];
  bool ok = ref_sh::TXValidate(&md, ts, r, rd, wr, hp, tp, oldhp, &st, 0, times);
  if (ok) return 0;
  return st.nbAbortsRecordAge ? 1 : 2;
}

/* plain TXAddToRecord for one transaction (no concurrent committers): returns the commit ts
 * (0 = abort) and the ring/metadata after the call */
uint32_t ref_sh_add_to_record(orc_record_c* recs, int* tp, int* r_hp, int* w_hp, int ts,
                              const uint32_t* rs, int nrs, const uint32_t* ws, int nws) {
  static ref_sh::TXRecord r[1600];
  static ref_sh::readSet rd[1];
  static ref_sh::writeSet wr[1];
  fill_sh_records(r, recs);
  rd[0].size = (ushort)nrs;
  for (int k = 0; k < nrs; k++) rd[0].addrs[k] = rs[k];
  wr[0].size = (ushort)nws;
  for (int k = 0; k < nws; k++) wr[0].addrs[k] = ws[k];
  ref_sh::TMmetadata md = {(ushort)*tp, (ushort)*r_hp, *w_hp};
  ref_sh::Statistics st;
  memset(&st, 0, sizeof(st));
  static ref_sh::time_rate times[1];
  int res = ref_sh::TXAddToRecord(&md, r, rd, wr, &st, times, ts, 0);
  *tp = md.tp;
  *r_hp = md.r_hp;
  *w_hp = md.w_hp;
  for (int i = 0; i < 1600; i++) {
    recs[i].txn = r[i].transactionNumber;
    recs[i].n_writes = r[i].n_writes;
    recs[i].ws[0] = r[i].writeSet[0];
    recs[i].ws[1] = r[i].writeSet[1];
  }
  return (uint32_t)res;
}

/* batched TXValidate; returns 0 valid, 1 RecordAge, 2 ReadWrite */
int ref_bt_validate(const orc_record_c* recs, int hp, int tp, int oldhp, int ts,
                    const uint32_t* rs, int nrs) {
  static ref_bt::TXRecord r[2000];
  static ref_bt::readSet rd;
  static ref_bt::writeSet wr;
  for (int i = 0; i < 2000; i++) {
    r[i].transactionNumber = recs[i].txn;
    r[i].n_writes = (ushort)recs[i].n_writes;
    r[i].writeSet[0] = recs[i].ws[0];
    r[i].writeSet[1] = recs[i].ws[1];
  }
  rd.size = (ushort)nrs;
  for (int k = 0; k < nrs; k++) rd.addrs[k] = rs[k];
  wr.size = 0;
  ref_bt::TMmetadata md;
  memset(&md, 0, sizeof(md));
  md.tp = (ushort)tp;
  md.r_hp = (ushort)hp;
  md.w_hp = hp;
  ref_bt::Statistics st;
  memset(&st, 0, sizeof(st));
  static ref_bt::time_rate times[1];
  bool ok = ref_bt::TXValidate(&md, ts, r, rd, wr, hp, oldhp, &st, 0, times);
  if (ok) return 0;
  return st.nbAbortsRecordAge ? 1 : 2;
}

/* TXPreValidation on a 32-lane warp; rs/ws are [32][stride]; returns the commit mask */
uint32_t ref_bt_prevalidate(const uint32_t* rs, const uint32_t* nrs, int rs_stride,
                            const uint32_t* ws, const uint32_t* nws, int ws_stride) {
  static ref_bt::readSet rd[32];
  static ref_bt::writeSet wr[32];
  for (int l = 0; l < 32; l++) {
    rd[l].size = (ushort)nrs[l];
    for (uint32_t k = 0; k < nrs[l]; k++) rd[l].addrs[k] = rs[l * rs_stride + k];
    wr[l].size = (ushort)nws[l];
    for (uint32_t k = 0; k < nws[l]; k++) {
      wr[l].addrs[k] = ws[l * ws_stride + k];
      wr[l].value[k] = 0;
    }
  }
  static bool res[32];
  run_warp([](unsigned l) { res[l] = ref_bt::TXPreValidation(l, rd, wr); });
  uint32_t m = 0;
  for (int l = 0; l < 32; l++)
    if (res[l]) m |= 1u << l;
  return m;
}

} /* extern "C" */
