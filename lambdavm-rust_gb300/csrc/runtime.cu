// runtime.cu — GB300 HVM2 runtime: turn kernel, fixed scheduling policy,
// host normalise/expand loop, readback, and the C ABI (`hvm_cu` and the
// handle API declared in include/hvm_gb300.h).
//
// Execution model (sm_103a, one GPU):
//   * One turn = one launch of `turn_kernel` over a grid sized to the SMs
//     (every resident block runs once). A thread takes its share of the
//     turn's input redexes from the global ring, then runs up to `budget`
//     interactions from its shared-memory LIFO, claiming more input from the
//     ring when its LIFO drains. Whatever is left, plus overflow, goes back to
//     the ring tail for the next turn. This replaces the reference's
//     evaluator/inbetween launch pair and its two blocking D2H copies per turn
//     (src/hvm.cu:1810-1839): the last block to finish computes the next
//     turn's input range and policy on the device, and the host only polls
//     the control block after a batch of turns.
//   * Termination: a turn that leaves no redex in the ring ends the
//     normalisation (the reference stops when the global bag is empty).
//   * The readback (`expand`, the lambda-encoded constructor walk of the IO
//     loop, src/run.cu:67-97 / src/hvm.cu:1861-1893) runs on the host over
//     single-word reads, and the final tree is serialised by one gather
//     kernel instead of a device printf (src/hvm.cu:2290-2297).
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <errno.h>
#include <time.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <mutex>
#include <vector>

#include "hvm_defs.h"
#include "evaluator.cuh"
#include "policy.cuh"
#include "hvm_gb300.h"

HVM_NS_BEGIN

// Capacity of each thread's page list (pages of one space a thread may own).
constexpr uint32_t MAX_PAGES = 64;
constexpr uint32_t HOST_NODE_WORDS = 1u << 21;  // node words the host may write IO results into (at most 1/64 of the space)
// IO encodings (src/run.c:32-60).
constexpr uint32_t IO_MAGIC_0 = 0xD0CA11, IO_MAGIC_1 = 0xFF1FF1;
constexpr uint32_t IO_CALL_TAG = 1;
constexpr uint32_t RESULT_OK_TAG = 0, RESULT_ERR_TAG = 1;
constexpr uint32_t IO_ERR_TYPE_TAG = 0, IO_ERR_NAME_TAG = 1, IO_ERR_INNER_TAG = 2;
constexpr uint32_t LIST_NIL_TAG = 0, LIST_CONS_TAG = 1;
constexpr uint32_t HOST_VAR_WORDS = 1u << 20;   // var words of the same
constexpr uint32_t LIST_READ_MAX = 1u << 20;    // list elements one device readback pass returns
// Batches: nets per batch (each takes one ROOT var at the top of the var
// space) and definitions over all nets (REF vals have 28 bits).
constexpr uint32_t MAX_BATCH = 1u << 20;
constexpr uint32_t MAX_BATCH_DEFS = 1u << 27;

static const char* status_text(uint32_t s) {
  switch (s) {
    case ST_OK: return "ok";
    case ST_OOM_NODES: return "out of node memory";
    case ST_OOM_VARS: return "out of var memory";
    case ST_RING_FULL: return "redex ring overflow";
    case ST_LINK_UNSET: return "link met an uninitialised var";
    case ST_LINK_LIMIT: return "substitution chain too long";
    case ST_BAD_REF: return "reference to a missing definition";
    case ST_DRAIN: return "local net not drained at the turn's end";
    case ST_WAIT: return "a persistent launch waited too long for a turn to close";
    default: return "unknown device error";
  }
}

// ---- turn kernel -------------------------------------------------------------------

__device__ __forceinline__ unsigned long long ldcg64(const unsigned long long* p) { return __ldcg(p); }

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  return v;
}

// Fixed work-distribution policy (the GB300 counterpart of the reference's
// SEED/GROW/WORK modes, src/hvm.cu:1509-1548). While the ring holds fewer
// redexes than threads, turns are short so fresh redexes spread over more
// threads each turn; if the ring stops growing (sequential work), the turn
// budget doubles so a lone chain is not cut into tiny turns. Once every
// thread has work, a turn runs until too many threads have run dry (`stop`),
// and its leftovers are then redistributed evenly.
__device__ void fixed_policy(Ctl* c, unsigned long long pending, unsigned long long prev_pending,
                             uint32_t nthreads, uint32_t cap) {
  uint32_t s, budget, chunk;
  if (pending < nthreads) {
    s = 1;
    chunk = 1;
    // Sequential or slowly growing work keeps doubling the budget; a jump in
    // the number of redexes (fresh parallelism) starts short turns again.
    uint32_t prev = c->budget;
    bool jump = pending > 2 * prev_pending + 64;
    budget = (!jump && prev >= 64) ? (prev < (1u << 16) ? prev * 2 : prev) : 64;
  } else {
    unsigned long long per = pending / nthreads;
    s = (uint32_t)(per < cap / 2 ? per : cap / 2);
    if (s == 0) s = 1;
    chunk = cap / 4 > 1 ? cap / 4 : 1;
    budget = 1u << 16;
  }
  unsigned long long busy = pending < nthreads ? pending : nthreads;
  unsigned long long keep = (busy * (256 - c->stop_frac_q8)) >> 8;  // busy threads that keep the turn going
  c->stop_at = (uint32_t)(nthreads - keep);
  c->static_per_thread = s;
  c->budget = c->budget_cap && budget > c->budget_cap ? c->budget_cap : budget;
  c->chunk = chunk;
}

// The scheduler's 16 inputs, computed by one thread from the control block at
// the close of a turn (all roughly in [0, 1]).
__device__ void policy_features(const Dev& d, unsigned long long pending, unsigned long long prev_pending,
                                float* f) {
  Ctl* c = d.ctl;
  const float N = (float)d.nthreads;
  unsigned long long now;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
  const float dt_us = c->turn_t0 ? (float)(now - c->turn_t0) * 1e-3f : 0.f;
  c->turn_t0 = now;
  const unsigned long long itrs = c->itrs, leak = c->leak;
  const float it = (float)(itrs - c->prev_itrs), lk = (float)(leak - c->prev_leak);
  float h[8];
  for (int i = 0; i < 8; i++) { h[i] = (float)(c->hist[i] - c->prev_hist[i]); c->prev_hist[i] = c->hist[i]; }
  c->prev_itrs = itrs;
  c->prev_leak = leak;
  const float P = (float)pending, Pp = (float)prev_pending;
  f[0] = log2f(1.f + P) / 24.f;
  f[1] = log2f(1.f + P / N) / 8.f;
  f[2] = log2f(1.f + Pp) / 24.f;
  f[3] = fminf(fmaxf(log2f((1.f + P) / (1.f + Pp)) / 8.f, -1.f), 1.f);
  f[4] = (float)c->dry / N;
  f[5] = c->stop ? 1.f : 0.f;
  f[6] = log2f(1.f + (float)c->budget) / 17.f;
  f[7] = log2f(1.f + it / N) / 8.f;
  f[8] = log2f(1.f + dt_us) / 20.f;
  f[9] = (float)c->live_nodes / (float)(d.node_mask + 1ull);
  f[10] = (float)c->live_vars / (float)(d.vars_mask + 1ull);
  f[11] = lk / (1.f + it);
  f[12] = log2f(1.f + (float)c->turns) / 16.f;
  f[13] = h[CALL] / (1.f + it);
  f[14] = h[ANNI] / (1.f + it);
  f[15] = (h[OPER] + h[SWIT]) / (1.f + it);
}

// Maps the policy's three outputs in [0, 1] onto the next turn, after the
// fixed policy has made its choice: o0 the budget (64 << round(10 o0), i.e.
// 64 .. 65536 rounds), o1 the stop fraction (32 + 192 o1, in 1/256), o2 the
// share of the input each thread takes statically (o2 * min(P/N, cap/2)) when
// every thread has work. A negative or non-finite output keeps the fixed
// choice. `eff` receives the parameters actually chosen, in the same space.
__device__ void apply_policy(Ctl* c, const float* o, unsigned long long pending, uint32_t nthreads, uint32_t cap,
                             float* eff) {
  unsigned long long busy = pending < nthreads ? pending : nthreads;
  if (o[0] >= 0.f && isfinite(o[0])) {
    const uint32_t b = 64u << (uint32_t)lrintf(fminf(o[0], 1.f) * 10.f);
    c->budget = c->budget_cap && b > c->budget_cap ? c->budget_cap : b;
  }
  uint32_t frac = c->stop_frac_q8;
  if (o[1] >= 0.f && isfinite(o[1])) {
    frac = 32u + (uint32_t)(fminf(o[1], 1.f) * 192.f);
    unsigned long long keep = (busy * (256 - frac)) >> 8;
    c->stop_at = (uint32_t)(nthreads - keep);
  }
  float share = 1.f;
  if (pending >= nthreads) {
    unsigned long long per = pending / nthreads;
    uint32_t full = (uint32_t)(per < cap / 2 ? per : cap / 2);
    if (full == 0) full = 1;
    if (o[2] >= 0.f && isfinite(o[2])) {
      uint32_t s = (uint32_t)lrintf(fminf(o[2], 1.f) * (float)full);
      c->static_per_thread = s ? s : 1;
    }
    share = (float)c->static_per_thread / (float)full;
  }
  eff[0] = log2f((float)(c->budget >> 6)) / 10.f;
  eff[1] = ((float)frac - 32.f) / 192.f;
  eff[2] = share;
}

// MIN_BLOCKS_128 > 0 asks the compiler to fit that many 128-thread blocks per
// SM (a register cap); the runtime picks the variant from the configuration.
// FAST compiles in the CALL-time fast paths (Dev::fast_calls), PROF the
// per-phase clock counters (Ctl::prof) and LOCAL the block-local nets
// (evaluator.cuh); each is kept out of the default variants because its code
// alone costs the others registers.
// The parameters of the turn about to run, read once per block so that every
// thread of the block takes the same decisions. Returns whether the turn has
// work (false: normal form reached, or a failure was recorded).
struct TurnParams {
  unsigned long long base, in_end;
  uint32_t s, budget, stop_at;
};
__device__ __forceinline__ bool turn_begin(const Dev& d, TurnParams& tp) {
  Ctl* c = d.ctl;
  __shared__ unsigned long long sh_base, sh_end;
  __shared__ unsigned sh_run, sh_s, sh_budget, sh_stop_at;
  if (threadIdx.x == 0) {
    sh_base = ldcg64(&c->base);
    sh_end = ldcg64(&c->in_end);
    sh_run = sh_base != sh_end && __ldcg(&c->status) == 0;
    sh_s = __ldcg(&c->static_per_thread);
    sh_budget = __ldcg(&c->budget);
    sh_stop_at = __ldcg(&c->stop_at);
  }
  __syncthreads();
  tp.base = sh_base;
  tp.in_end = sh_end;
  tp.s = sh_s;
  tp.budget = sh_budget;
  tp.stop_at = sh_stop_at;
  const bool run = sh_run != 0;
  __syncthreads();  // the shared words are rewritten by the next turn's call
  return run;
}

// One turn's work for this block: static share of the input, rounds until
// the budget or the stop flag, LIFO flush to the ring tail, counters.
template <int MIN_BLOCKS_128, bool FAST, bool PROF, bool LOCAL>
__device__ __forceinline__ void turn_work(const Dev& d, uint32_t cap, const TurnParams& tp) {
  extern __shared__ unsigned long long smem_stack[];
  Ctl* c = d.ctl;
  const unsigned long long base = tp.base, in_end = tp.in_end;
  const uint32_t s = tp.s, budget = tp.budget, stop_at = tp.stop_at;

  TState t;
  t.stk = (Pair*)smem_stack + threadIdx.x;
  t.stride = blockDim.x;
  t.lo = 0;
  t.len = 0;
  t.cap = cap;
  t.gid = blockIdx.x * blockDim.x + threadIdx.x;
  alloc_load<false>(d.nspace, t.gid, t.na);
  alloc_load<true>(d.vspace, t.gid, t.va);
  t.base = base;
  t.itrs = t.leak = t.retries = 0;
  t.live_nodes = t.live_vars = 0;
  t.dirty = false;
  for (int i = 0; i < 8; i++) t.hist[i] = 0;
  t.dead = false;
  t.waited = 0;
  if (LOCAL) {
    // Each lane clears its own slice of the block's local net (128-thread blocks).
    for (uint32_t i = 0; i < LOCAL_SLICE; i++) { lnode_of(t)[lbase_of() + i] = 0; lvar_of(t)[lbase_of() + i] = 0; }
    ovf_len_of(t) = 0;
  }

  // Static share of the input: items base + gid + k*N, k < s.
  for (uint32_t k = 0; k < s; k++) {
    unsigned long long at = base + t.gid + (unsigned long long)k * d.nthreads;
    if (at >= in_end) break;
    push<LOCAL>(d, t, ring_pair(&d.ring[at & d.ring_mask]));
  }

  const unsigned lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1;
  Pair* warp_stk = t.stk - lane;  // lane j's deque starts at warp_stk + j
  WarpProf prof;
  const bool prof_on = PROF && __ldcg(&c->prof_on) != 0;
  for (int i = 0; i < 8; i++) prof.v[i] = 0;
  long long t_loop = clock64();
  // The turn's input is [base, in_end) and `head` only grows: once a claim
  // finds it exhausted, the warp stops polling it (an L2 round trip a round).
  bool ring_dry = false;
  unsigned stop_flag = 0;  // lane 0: the stop flag as loaded after the previous round
  for (uint32_t round = 0; round < budget; round++) {
    // Intra-warp balancing: each empty lane takes the oldest redex of a lane
    // holding two or more (all in shared memory, no global traffic).
    unsigned want = __ballot_sync(0xFFFFFFFFu, t.len == 0);
    unsigned give = __ballot_sync(0xFFFFFFFFu, t.len >= d.steal_min);
    if (want && give) {
      // A giving lane whose fresh words are not yet fenced publishes them
      // before another lane can take a redex that points at them.
      if (__any_sync(0xFFFFFFFFu, ((give >> lane) & 1) && t.dirty)) { __threadfence(); t.dirty = false; }
      unsigned m = min(__popc(want), __popc(give));
      unsigned rw = __popc(want & lt_mask), rg = __popc(give & lt_mask);
      bool recv = ((want >> lane) & 1) && rw < m;
      int donor = recv ? (int)__fns(give, 0, rw + 1) : (int)lane;
      unsigned dlo = __shfl_sync(0xFFFFFFFFu, t.lo, donor);
      Pair got = recv ? warp_stk[(size_t)dlo * t.stride + donor] : 0;
      __syncwarp();
      if (((give >> lane) & 1) && rg < m) { t.lo = (t.lo + 1) & (t.cap - 1); t.len--; }
      if (recv) push<LOCAL>(d, t, got);
    }
    // Local-net variant: a lane's own spilled redexes come back first.
    if (LOCAL && t.len == 0 && ovf_len_of(t) > 0) push<LOCAL>(d, t, ovf_of(d, t)[--ovf_len_of(t)]);
    // Lanes still empty claim ring input, one atomic for the warp.
    unsigned empty = __ballot_sync(0xFFFFFFFFu, t.len == 0);
    if (empty && !ring_dry) {
      unsigned long long h = 0;
      if (lane == 0) {
        h = ldcg64(&c->head);
        if (h < in_end) h = atomicAdd(&c->head, (unsigned long long)__popc(empty));
      }
      h = __shfl_sync(0xFFFFFFFFu, h, 0);
      unsigned k = __popc(empty & lt_mask);
      if (((empty >> lane) & 1) && h + k < in_end) {
        push<LOCAL>(d, t, ring_pair(&d.ring[(h + k) & d.ring_mask]));
      }
      ring_dry = h + __popc(empty) >= in_end;
    }
    if (!__any_sync(0xFFFFFFFFu, t.len > 0)) {
      // The whole warp ran dry: count it; enough dry threads end the turn.
      if (lane == 0) {
        unsigned g = atomicAdd(&c->dry, 32u) + 32;
        if (g >= stop_at) atomicExch(&c->stop, 1u);
      }
      break;
    }
    // Rule selection (d.rule_select != 0): the warp runs one class of rules
    // per round -- the class of the most lanes' next redex, or of a lane that
    // has waited RULE_WAIT_MAX rounds -- and the other lanes keep their
    // redex for a later round, so only that class's code path executes.
    bool go = t.len > 0;
    if (d.rule_select) {
      const uint32_t cls = go ? rule_class(d.rule_select, slot(t, t.len - 1)) : 0xFFu;
      const unsigned same = __match_any_sync(0xFFFFFFFFu, cls);
      unsigned key = 0;
      if (go) key = (t.waited >= RULE_WAIT_MAX ? 1u << 12 : 0u) | ((unsigned)__popc(same) << 5) | (31u - lane);
      key = __reduce_max_sync(0xFFFFFFFFu, key);
      const uint32_t chosen = __shfl_sync(0xFFFFFFFFu, cls, 31u - (key & 31u));
      const bool run = go && cls == chosen;
      t.waited = run || !go ? 0 : t.waited + 1;
      go = run;
    }
    const bool has = go;
    const Pair r = has ? pop(t) : 0;
    lockstep_round<FAST, LOCAL, MIN_BLOCKS_128 != 8>(d, t, has, r, prof_on ? &prof : nullptr);
    if (__any_sync(0xFFFFFFFFu, t.dead)) break;
    if (LOCAL && __any_sync(0xFFFFFFFFu, ovf_len_of(t) > OVF_HIGH)) break;  // end the turn before an overflow fills
    // The stop flag is tested one round after it was loaded, so its L2
    // latency hides behind a whole round (a short round would otherwise wait
    // for it).
    if (__shfl_sync(0xFFFFFFFFu, stop_flag, 0)) break;
    if (lane == 0) stop_flag = *(volatile unsigned*)&c->stop;
  }

  if (LOCAL) {
    // Turn's end: every redex this lane holds that names local words is
    // made global (GLOBALIZE; LEAK for the local nodes it reaches), the
    // others go to the ring as they are; the block's local net then ends.
    // A lane holds at most OVF_CAP + cap redexes and its block at most
    // LOCAL_WORDS local nodes, each leaked once: the bound is generous.
    for (uint32_t guard = 0;; guard++) {
      if (t.len == 0 && ovf_len_of(t) > 0) push<LOCAL>(d, t, ovf_of(d, t)[--ovf_len_of(t)]);
      bool has = t.len > 0 && !t.dead;
      if (!__any_sync(0xFFFFFFFFu, has)) break;
      if (guard >= (1u << 16)) {
        if (lane == 0) set_status(d, ST_DRAIN, t.gid);
        break;
      }
      const Pair r = has ? pop(t) : 0;
      if (has && !local_pair(r)) { ring_put(d, t, r); has = false; }
      lockstep_round<FAST, LOCAL, MIN_BLOCKS_128 != 8>(d, t, has, r, nullptr, true);
      if (__any_sync(0xFFFFFFFFu, t.dead)) break;
    }
  }

  if (prof_on && lane == 0) {
    prof.v[PROF_CYC_ROUND] = clock64() - t_loop;  // whole loop, including balancing and claims
    for (int i = 0; i < 8; i++) if (prof.v[i]) atomicAdd(&c->prof[i], prof.v[i]);
  }
  alloc_save(d.nspace, t.gid, t.na);
  alloc_save(d.vspace, t.gid, t.va);

  // Flush the LIFO to the ring tail, one atomic per warp.
  __syncwarp();
  uint32_t n = t.len, incl = n;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (unsigned)o) incl += y;
  }
  uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  unsigned long long wbase = 0;
  if (lane == 31 && total) wbase = atomicAdd(&c->tail, (unsigned long long)total);
  wbase = __shfl_sync(0xFFFFFFFFu, wbase, 31);
  if (total) {
    unsigned long long my = wbase + incl - n;
    if (wbase + total - base > d.ring_mask + 1) {
      if (lane == 0) set_status(d, ST_RING_FULL, 1);
    } else {
      for (uint32_t i = 0; i < n; i++) d.ring[(my + i) & d.ring_mask] = slot(t, i);
      t.leak += n;
    }
  }

  // Counters: reduced per warp, then per block in shared memory, then one
  // global atomic per counter per block.
  // Live-word deltas: one atomic per warp.
  {
    long long ln = t.live_nodes, lv = t.live_vars;
    for (int o = 16; o > 0; o >>= 1) {
      ln += __shfl_down_sync(0xFFFFFFFFu, ln, o);
      lv += __shfl_down_sync(0xFFFFFFFFu, lv, o);
    }
    if (lane == 0 && ln) atomicAdd((unsigned long long*)&c->live_nodes, (unsigned long long)ln);
    if (lane == 0 && lv) atomicAdd((unsigned long long*)&c->live_vars, (unsigned long long)lv);
  }
  __shared__ unsigned long long blk_cnt[11];
  if (threadIdx.x < 11) blk_cnt[threadIdx.x] = 0;
  __syncthreads();
  unsigned long long v;
  v = warp_sum(t.itrs);    if (lane == 0 && v) atomicAdd(&blk_cnt[0], v);
  v = warp_sum(t.leak);    if (lane == 0 && v) atomicAdd(&blk_cnt[1], v);
  v = warp_sum(t.retries); if (lane == 0 && v) atomicAdd(&blk_cnt[2], v);
  for (int i = 0; i < 8; i++) {
    v = warp_sum(t.hist[i]);
    if (lane == 0 && v) atomicAdd(&blk_cnt[3 + i], v);
  }
  __syncthreads();
  if (threadIdx.x < 11 && blk_cnt[threadIdx.x]) {
    unsigned long long* dst = threadIdx.x == 0 ? &c->itrs : threadIdx.x == 1 ? &c->leak
                            : threadIdx.x == 2 ? &c->retries : &c->hist[threadIdx.x - 3];
    atomicAdd(dst, blk_cnt[threadIdx.x]);
  }

}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// The last block to finish closes the turn and picks the next one. In a
// persistent launch (PERSIST) every block arrives, also one whose turn had
// no work, and the closing block decides whether the launch goes on: turn
// `k` of `turns`, while the pending count stays in [lo, hi) (outside it the
// host switches kernel variants), no failure recorded and redexes left.
template <bool PERSIST>
__device__ __forceinline__ void turn_close(const Dev& d, uint32_t cap, const TurnParams& tp, bool ran, uint32_t k,
                                           uint32_t turns, unsigned long long lo, unsigned long long hi) {
  Ctl* c = d.ctl;
  const unsigned long long in_end = tp.in_end;
  __shared__ unsigned sh_last;
  __shared__ float feat[POLICY_IN], h1[POLICY_HID], h2[POLICY_HID], outp[POLICY_OUT];
  __shared__ unsigned long long sh_pending, sh_prev, sh_nb, sh_tail;
  __syncthreads();
  if (PERSIST && threadIdx.x == 0 && !ran) {
    // Nothing ran in this block: arrive; the closing block (if it is this
    // one) only lets the launch end.
    __threadfence();
    const unsigned prev = atomicAdd(&c->blocks_done, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      c->go = 0;
      c->persist_ran = k;
      c->blocks_done = 0;
      __threadfence();
      st_release_u32(&c->epoch, ld_acquire_u32(&c->epoch) + 1);
    }
  }
  if (PERSIST && !ran) return;
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned prev = atomicAdd(&c->blocks_done, 1u);
    sh_last = prev == gridDim.x - 1;
    if (sh_last) {
      __threadfence();
      unsigned long long head = ldcg64(&c->head), tail = ldcg64(&c->tail);
      sh_nb = head < in_end ? head : in_end;
      sh_tail = tail;
      sh_pending = tail - sh_nb;
      sh_prev = c->pending;
      policy_features(d, sh_pending, sh_prev, feat);
    }
  }
  __syncthreads();
  if (!sh_last) return;
  const uint32_t mode = __ldcg(&c->policy_mode);
  if (mode == POLICY_LEARNED && c->policy_w) policy_infer_block(c->policy_w, feat, h1, h2, outp);
  if (threadIdx.x == 0) {
    const unsigned long long pending = sh_pending, prev_pending = sh_prev, nb = sh_nb;
    if (mode == POLICY_CONSTANT) {
      const int k = pending < d.nthreads ? 0 : 3;
      outp[0] = c->policy_const[k]; outp[1] = c->policy_const[k + 1]; outp[2] = c->policy_const[k + 2];
    } else if (mode == POLICY_SCRIPT) {
      const unsigned long long k = c->turns;  // the turn being closed
      const bool in = c->policy_w && k < c->policy_script_len;
      for (int o = 0; o < POLICY_OUT; o++) outp[o] = in ? c->policy_w[3 * k + o] : -1.f;
    } else if (mode != POLICY_LEARNED || !c->policy_w) {
      outp[0] = outp[1] = outp[2] = -1.f;
    }
    float eff[POLICY_OUT];
    const unsigned closed_budget = c->budget, closed_share = c->static_per_thread;
    const unsigned closed_dry = c->dry, closed_stop = c->stop;
    const unsigned long long closed_turn = c->turns;
    c->base = nb;
    c->in_end = sh_tail;
    c->pending = pending;
    c->turns += 1;
    c->dry = 0;
    c->stop = 0;
    // Free-page rings: the pages returned this turn become takeable.
    c->nf_head = c->nf_head < c->nf_end ? c->nf_head : c->nf_end;
    c->nf_end = c->nf_tail;
    c->vf_head = c->vf_head < c->vf_end ? c->vf_head : c->vf_end;
    c->vf_end = c->vf_tail;
    fixed_policy(c, pending, prev_pending, d.nthreads, cap);
    apply_policy(c, outp, pending, d.nthreads, cap, eff);
    if (c->trace && closed_turn < c->trace_cap) {
      unsigned long long now;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
      TurnRecord r;
      r.t_ns = now;
      r.live_nodes = c->live_nodes;
      r.itrs = c->itrs;
      r.pending = pending;
      r.dry = closed_dry;
      r.stopped = closed_stop;
      r.budget = closed_budget;
      r.per_thread = closed_share;
      for (int i = 0; i < POLICY_IN; i++) r.features[i] = feat[i];
      for (int i = 0; i < POLICY_OUT; i++) r.outputs[i] = eff[i];
      c->trace[closed_turn] = r;
    }
    unsigned long long take = (unsigned long long)c->static_per_thread * d.nthreads;
    c->head = nb + (take < pending ? take : pending);
    c->blocks_done = 0;
    __threadfence();
    if (PERSIST) {
      c->go = c->status == 0 && pending != 0 && k + 1 < turns && pending >= lo && pending < hi;
      c->persist_ran = k + 1;
      __threadfence();
      st_release_u32(&c->epoch, ld_acquire_u32(&c->epoch) + 1);
    }
  }
}

template <int MIN_BLOCKS_128, bool FAST, bool PROF, bool LOCAL>
__global__ void __launch_bounds__(128, MIN_BLOCKS_128 > 0 ? MIN_BLOCKS_128 : 1) turn_kernel(Dev d, uint32_t cap) {
  TurnParams tp;
  if (!turn_begin(d, tp)) return;
  turn_work<MIN_BLOCKS_128, FAST, PROF, LOCAL>(d, cap, tp);
  turn_close<false>(d, cap, tp, true, 0, 0, 0, 0);
}

// Longest wait of a persistent launch's block for a turn to close; a turn is
// bounded by its round budget and takes milliseconds.
constexpr unsigned long long PERSIST_WAIT_NS = 2000000000ull;
// Turns per persistent launch: the host polls between launches (progress
// and turn-budget checks, kernel-variant switches).
constexpr uint32_t PERSIST_TURNS = 4096;

// Waits until *p differs from `v`, for at most `limit_ns` of the global
// timer; returns false if the limit ran out.
__device__ __forceinline__ bool wait_change(const unsigned* p, unsigned v, unsigned long long limit_ns) {
  unsigned long long t0, now;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (uint32_t spin = 0; ld_acquire_u32(p) == v; spin++) {
    __nanosleep(200);
    if ((spin & 1023) == 1023) {
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
      if (now - t0 > limit_ns) return false;
    }
  }
  return true;
}

// Self-test of the wait: one thread waits on a word that nothing writes and
// reports (out[0]) whether the limit ran out and (out[1..2]) the time waited.
__global__ void wait_probe_kernel(const unsigned* word, unsigned long long limit_ns, unsigned* out) {
  unsigned long long t0, t1;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  const bool changed = wait_change(word, *word, limit_ns);
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
  out[0] = changed ? 0u : 1u;
  out[1] = (unsigned)((t1 - t0) & 0xFFFFFFFFu);
  out[2] = (unsigned)((t1 - t0) >> 32);
}

// Persistent launch (cooperative, so every block is resident): up to `turns`
// turns in one launch, each closed on the device as turn_kernel's are; the
// blocks that did not close a turn wait for its epoch, with a time limit
// after which they record ST_WAIT and return.
template <int MIN_BLOCKS_128>
__global__ void __launch_bounds__(128, MIN_BLOCKS_128 > 0 ? MIN_BLOCKS_128 : 1)
    persistent_kernel(Dev d, uint32_t cap, uint32_t turns, unsigned long long lo, unsigned long long hi) {
  Ctl* c = d.ctl;
  __shared__ unsigned sh_go;
  // No turn closes before every block has arrived at the first close, so
  // every block reads the same starting epoch.
  const unsigned e0 = ld_acquire_u32(&c->epoch);
  for (uint32_t k = 0; k < turns; k++) {
    TurnParams tp;
    const bool ran = turn_begin(d, tp);
    if (ran) turn_work<MIN_BLOCKS_128, false, false, false>(d, cap, tp);
    turn_close<true>(d, cap, tp, ran, k, turns, lo, hi);
    if (threadIdx.x == 0) {
      const bool late = !wait_change(&c->epoch, e0 + k, PERSIST_WAIT_NS);
      if (late) set_status(d, ST_WAIT, blockIdx.x);
      sh_go = late ? 0u : __ldcg(&c->go);
    }
    __syncthreads();
    if (!sh_go) return;
  }
}

// Gives thread g page g of each space (past the reserved first pages, whose
// indices the local-net variant uses) and points both pools past them.
__global__ void reset_alloc_kernel(Dev d) {
  uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < d.nthreads) {
    for (const PagedSpace* sp : {&d.nspace, &d.vspace}) {
      sp->lists[(size_t)g * sp->max_pages] = g + (sp == &d.nspace ? d.npool_base : d.vpool_base);
      sp->counts[g] = 1;
      sp->pos[g] = 0;
      sp->off[g] = 0;
    }
  }
  if (g == 0) {
    d.ctl->npool_next = d.nthreads + d.npool_base;
    d.ctl->vpool_next = d.nthreads + d.vpool_base;
  }
}

// Starts a normalisation from `redex` (src/hvm.cu:1488-1497): sets the root
// var (ROOT, or net k's ROOT var in a batch) to NONE and makes `redex` the
// only input of the next turn.
__global__ void boot_kernel(Dev d, Pair redex, Port root, uint32_t cap) {
  Ctl* c = d.ctl;
  if (get_tag(root) == VAR) d.vars[get_val(root) & d.vars_mask] = NONE;
  unsigned long long at = c->tail;
  d.ring[at & d.ring_mask] = redex;
  c->base = at;
  c->in_end = at + 1;
  c->tail = at + 1;
  c->pending = 1;
  c->blocks_done = 0;
  c->dry = 0;
  c->stop = 0;
  c->budget = 0;
  fixed_policy(c, 1, 1, d.nthreads, cap);
  c->head = at + 1;
  __threadfence();
}

// Re-plans the next turn for a grid of d.nthreads threads after the host
// switched kernel variants between two turns: the static share, the claim
// head and the stop threshold depend on the thread count (as fixed_policy
// sets them); the round budget is kept.
__global__ void retarget_kernel(Dev d, uint32_t cap) {
  Ctl* c = d.ctl;
  const unsigned long long pending = c->in_end - c->base;
  const uint32_t n = d.nthreads;
  uint32_t s = 1;
  if (pending >= n) {
    unsigned long long per = pending / n;
    s = (uint32_t)(per < cap / 2 ? per : cap / 2);
    if (s == 0) s = 1;
  }
  unsigned long long busy = pending < n ? pending : n;
  unsigned long long keep = (busy * (256 - c->stop_frac_q8)) >> 8;
  c->stop_at = (uint32_t)(n - keep);
  c->static_per_thread = s;
  c->chunk = pending < n ? 1 : (cap / 4 > 1 ? cap / 4 : 1);
  unsigned long long take = (unsigned long long)s * n;
  c->head = c->base + (take < pending ? take : pending);
  __threadfence();
}

// Starts a batch: net k's redex `@main_k ~ ROOT_k` with ROOT_k = ROOT_VAR - k.
__global__ void boot_batch_kernel(Dev d, const uint32_t* mains, uint32_t n, uint32_t cap) {
  Ctl* c = d.ctl;
  const unsigned long long at = c->tail;
  for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
    d.vars[(ROOT_VAR - k) & d.vars_mask] = NONE;
    d.ring[(at + k) & d.ring_mask] = new_pair(new_port(REF, mains[k]), new_port(VAR, ROOT_VAR - k));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    c->base = at;
    c->in_end = at + n;
    c->tail = at + n;
    c->pending = n;
    c->blocks_done = 0;
    c->dry = 0;
    c->stop = 0;
    c->budget = 0;
    fixed_policy(c, n, n, d.nthreads, cap);
    unsigned long long take = (unsigned long long)c->static_per_thread * d.nthreads;
    c->head = at + (take < n ? take : n);
    __threadfence();
  }
}

// Admits nets nets[0..k) of a loaded batch between two turns: each
// one's `@main ~ ROOT_net` joins the next turn's input, and the turn
// parameters are recomputed for the larger input.
__global__ void admit_kernel(Dev d, const uint32_t* mains, const uint32_t* nets, uint32_t k, uint32_t cap) {
  Ctl* c = d.ctl;
  const unsigned long long at = c->tail;
  for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) {
    uint32_t net = nets[i];
    d.vars[(ROOT_VAR - net) & d.vars_mask] = NONE;
    d.ring[(at + i) & d.ring_mask] = new_pair(new_port(REF, mains[net]), new_port(VAR, ROOT_VAR - net));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long prev = c->pending;
    c->tail = at + k;
    c->in_end = at + k;
    c->pending = c->in_end - c->base;
    c->blocks_done = 0;
    c->dry = 0;
    c->stop = 0;
    fixed_policy(c, c->pending, prev, d.nthreads, cap);
    unsigned long long take = (unsigned long long)c->static_per_thread * d.nthreads;
    c->head = c->base + (take < c->pending ? take : c->pending);
    __threadfence();
  }
}

// out[i] = net nets[i]'s ROOT with its var chain resolved (read-only).
__global__ void active_roots_kernel(Dev d, const uint32_t* nets, Port* out, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Port p = new_port(VAR, ROOT_VAR - nets[i]);
  for (uint32_t g = 0; g < (1u << 20) && get_tag(p) == VAR; g++) {
    Port v = __ldcg(&d.vars[get_val(p) & d.vars_mask]);
    if (v == NONE || v == 0) break;
    p = v;
  }
  out[i] = p;
}

// out[k] = net k's ROOT with its var chain resolved (read-only).
__global__ void batch_roots_kernel(Dev d, Port* out, uint32_t n) {
  uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  Port p = new_port(VAR, ROOT_VAR - k);
  for (uint32_t g = 0; g < (1u << 20) && get_tag(p) == VAR; g++) {
    Port v = __ldcg(&d.vars[get_val(p) & d.vars_mask]);
    if (v == NONE || v == 0) break;
    p = v;
  }
  out[k] = p;
}

// Counts live words of the net (the reference's count_memory debug kernel,
// src/hvm.cu:2234-2255): out[0] += non-zero node words, out[1] += non-zero
// var words, out[2] += node words still marked as taken-but-unwritten.
__global__ void count_live_kernel(Dev d, uint64_t n_nodes, uint64_t n_vars, unsigned long long* out) {
  unsigned long long a = 0, b = 0, m = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_nodes; i += (uint64_t)gridDim.x * blockDim.x) {
    Pair v = d.node[i];
    a += v != 0;
    m += v == NODE_MARK;
  }
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_vars; i += (uint64_t)gridDim.x * blockDim.x) {
    b += d.vars[i] != 0;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xFFFFFFFFu, a, o);
    b += __shfl_down_sync(0xFFFFFFFFu, b, o);
    m += __shfl_down_sync(0xFFFFFFFFu, m, o);
  }
  if ((threadIdx.x & 31) == 0) { atomicAdd(&out[0], a); atomicAdd(&out[1], b); atomicAdd(&out[2], m); }
}

// Serialises the tree reachable from `root` in breadth-first order:
// out[k] is a port with its var chain resolved; for a node port, kids[k] is
// the index of its first child (the second child follows it). One block.
__global__ void gather_kernel(Dev d, Port root, Port* out, uint32_t* kids, uint32_t cap, uint32_t* info) {
  __shared__ uint32_t next, lo, hi, overflow;
  auto resolve = [&](Port p) -> Port {
    for (uint32_t g = 0; g < (1u << 20) && get_tag(p) == VAR; g++) {
      Port v = __ldcg(&d.vars[get_val(p) & d.vars_mask]);
      if (v == NONE || v == 0) break;
      p = v;
    }
    return p;
  };
  if (threadIdx.x == 0) {
    out[0] = resolve(root);
    next = 1; lo = 0; hi = 1; overflow = 0;
  }
  __syncthreads();
  while (lo < hi && !overflow) {
    for (uint32_t k = lo + threadIdx.x; k < hi; k += blockDim.x) {
      Port p = out[k];
      if (is_nod(p)) {
        uint32_t pos = atomicAdd(&next, 2u);
        if (pos + 2 > cap) { overflow = 1; continue; }
        Pair nd = nload(d, (uint32_t)get_val(p));
        out[pos] = resolve(get_fst(nd));
        out[pos + 1] = resolve(get_snd(nd));
        kids[k] = pos;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) { lo = hi; hi = next < cap ? next : cap; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { info[0] = next < cap ? next : cap; info[1] = overflow; }
}

// Reads a lambda-encoded list of u24 (lam t (((t CONS) head) tail) ... lam t
// (t NIL)) straight from the net, as the host readback would, as long as no
// REF must be expanded (expansion normalises, which only the host loop
// does). info = {elements read, 1 if the host must continue, the port of the
// element where it stopped}. One thread: the list is a chain.
__global__ void read_list_kernel(Dev d, Port p, uint32_t max, uint32_t* out, uint32_t* info) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  auto peekp = [&](Port q) -> Port {
    for (uint32_t g = 0; g < (1u << 20) && get_tag(q) == VAR; g++) {
      Port v = __ldcg(&d.vars[get_val(q) & d.vars_mask]);
      if (v == NONE || v == 0) break;
      q = v;
    }
    return q;
  };
  auto node = [&](Port q) -> Pair { return nload(d, (uint32_t)get_val(q)); };
  uint32_t k = 0, host = 0;
  while (k < max) {
    const Port lam = peekp(p);
    if (get_tag(lam) == REF) { host = 1; break; }
    if (get_tag(lam) != CON) break;
    const Pair ln = node(lam);
    const Port app = peekp(get_fst(ln));
    if (get_tag(app) == REF) { host = 1; break; }
    if (get_tag(app) != CON) break;
    const Pair an = node(app);
    const Port tag = peekp(get_fst(an));
    if (get_tag(tag) == REF) { host = 1; break; }
    if (get_tag(tag) != NUM || get_u24(get_val(tag)) != 1) break;  // not a CONS
    const Port a1 = peekp(get_snd(an));
    if (get_tag(a1) == REF) { host = 1; break; }
    if (get_tag(a1) != CON) break;
    const Pair n1 = node(a1);
    const Port head = peekp(get_fst(n1)), a2 = peekp(get_snd(n1));
    if (get_tag(head) == REF || get_tag(a2) == REF) { host = 1; break; }
    if (get_tag(a2) != CON) break;
    const Pair n2 = node(a2);
    const Port tail = peekp(get_fst(n2)), a3 = peekp(get_snd(n2));
    if (get_tag(tail) == REF || get_tag(a3) == REF) { host = 1; break; }
    if (get_tag(a3) == CON || get_tag(head) != NUM) break;  // not exactly two arguments, or not a number
    out[k++] = get_u24(get_val(head));
    p = tail;
  }
  if (k == max) host = 1;
  info[0] = k;
  info[1] = host;
  info[2] = (uint32_t)p;  // the port where the host loop takes over, low and high words
  info[3] = (uint32_t)((uint64_t)p >> 32);
}

// ---- host runtime ----------------------------------------------------------------

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { return fail(std::string(#x) + ": " + cudaGetErrorString(e_)); } } while (0)

struct HostDef {
  std::string name;
  bool safe;
  uint32_t rbag_len, node_len, vars_len;
  Port root;
  std::vector<Pair> rbag, node;
};

// A CALL wires the def's redexes and then its root to the caller's port
// (src/hvm.c:865-898), each by the linker. Before upload, every def's links
// are rewritten as one list -- the redexes, then (root ~ CALLER_PORT) -- and
// a var whose two occurrences are both link ends (never inside a node) is
// removed by joining its two links: (P ~ v), (v ~ Q) become (P ~ Q). Such a
// var is only a wire between two links of the same call, so the device need
// not allocate, publish and take it (two atomic exchanges and a fence). The
// remaining vars are renumbered densely. Interactions and normal forms are
// unchanged: the same redexes are formed, only without the detour.
// Scratch buffers of join_links, reused from def to def (a book may hold
// thousands of defs; their loading is on the host's critical path).
struct JoinScratch {
  struct L { Port x, y; bool live; };
  std::vector<L> ls;
  std::vector<uint8_t> in_node;
  std::vector<uint32_t> map;
};

static void join_links(const HostDef& h, std::vector<Pair>& links, std::vector<Pair>& nodes, uint32_t& vars_len,
                       JoinScratch& sc) {
  using L = JoinScratch::L;
  std::vector<L>& ls = sc.ls;
  ls.clear();
  for (Pair p : h.rbag) ls.push_back({get_fst(p), get_snd(p), true});
  ls.push_back({h.root, CALLER_PORT, true});
  std::vector<uint8_t>& in_node = sc.in_node;
  in_node.assign(h.vars_len, 0);
  for (Pair p : h.node)
    for (Port q : {get_fst(p), get_snd(p)})
      if (get_tag(q) == VAR) in_node[get_val(q)] = 1;
  auto is_free_var = [&](Port q) { return q != CALLER_PORT && get_tag(q) == VAR && !in_node[get_val(q)]; };
  for (bool changed = true; changed;) {
    changed = false;
    for (size_t j = 0; j < ls.size() && !changed; j++) {
      if (!ls[j].live) continue;
      for (int side = 0; side < 2 && !changed; side++) {
        Port v = side ? ls[j].y : ls[j].x;
        if (!is_free_var(v)) continue;
        Port keep = side ? ls[j].x : ls[j].y;
        if (keep == v) continue;  // v ~ v: a closed loop, left to the linker
        for (size_t k = 0; k < ls.size(); k++) {
          if (k == j || !ls[k].live) continue;
          Port other;
          if (ls[k].x == v) other = ls[k].y;
          else if (ls[k].y == v) other = ls[k].x;
          else continue;
          ls[j] = {keep, other, true};
          ls[k].live = false;
          changed = true;
          break;
        }
      }
    }
  }
  // Dense renumbering of the vars still in use.
  std::vector<uint32_t>& map = sc.map;
  map.assign(h.vars_len, ~0u);
  uint32_t next = 0;
  auto renum = [&](Port q) -> Port {
    if (q == CALLER_PORT || get_tag(q) != VAR) return q;
    uint32_t& m = map[get_val(q)];
    if (m == ~0u) m = next++;
    return new_port(VAR, m);
  };
  links.clear();
  nodes.clear();
  for (Pair p : h.node) nodes.push_back(new_pair(renum(get_fst(p)), renum(get_snd(p))));
  for (const L& l : ls)
    if (l.live) links.push_back(new_pair(renum(l.x), renum(l.y)));
  vars_len = next;
}

// The CALL-time fast paths a def allows (DefHdr::fast). The reference's
// compiled C mode checks, at each call, whether the caller's port already
// has the shape the def's root would interact with (src/cmp.rs:110-290):
// a root CON meeting a CON node is annihilated on the spot, and a root
// `(?((s1 s2) r) r)` meeting `(#X R)` is switched on the spot, adding the
// interactions it performs (1, and 3) by hand. Only the top-level pattern is
// taken here; the def's other nodes are created as in any call. Needs the
// root link last in the joined link list, and fields of 5 bits.
static uint32_t fast_word(const HostDef& h, const std::vector<Pair>& links, const std::vector<Pair>& nodes,
                          uint32_t vars_len) {
  if (get_tag(h.root) != CON || h.node_len > 32 || vars_len > 32 || links.empty()) return 0;
  if (links.back() != new_pair(h.root, CALLER_PORT)) return 0;
  const uint32_t ri = get_val(h.root);
  const Port a1 = get_fst(nodes[ri]), a2 = get_snd(nodes[ri]);
  uint32_t w = FAST_ANNI | ri << 2;
  if (get_tag(a1) == SWI && get_tag(a2) == VAR) {
    const Pair sw = nodes[get_val(a1)];
    const Port a11 = get_fst(sw), a12 = get_snd(sw);
    if (get_tag(a11) == CON && a12 == a2)
      w = FAST_SWITCH | ri << 2 | get_val(a1) << 7 | get_val(a11) << 12 | get_val(a2) << 17;
  }
  return w;
}

// The device's def tables for a book: per def a header, then its links (the
// redexes and the root link, joined) and its nodes (and, for a def with a
// fast path, its two pairs of fast-path ports), all defs in one array.
static void def_tables(const std::vector<HostDef>& defs, std::vector<DefHdr>& hdr, std::vector<Pair>& flat,
                       uint32_t& max_nodes, uint32_t& max_vars) {
  hdr.assign(defs.size(), DefHdr{});
  flat.clear();
  size_t words = 1;
  for (const HostDef& h : defs) words += h.rbag.size() + 3 + h.node.size();
  flat.reserve(words);
  max_nodes = 1;
  max_vars = 1;
  JoinScratch sc;
  std::vector<Pair> links, nodes;
  for (size_t f = 0; f < defs.size(); f++) {
    const HostDef& h = defs[f];
    uint32_t vars_len = 0;
    join_links(h, links, nodes, vars_len, sc);
    const uint32_t fast = fast_word(h, links, nodes, vars_len);
    hdr[f] = DefHdr{h.node_len, (uint32_t)links.size(), vars_len, h.safe ? 1u : 0u, 0, (uint32_t)flat.size(), 1, fast};
    flat.insert(flat.end(), links.begin(), links.end());
    flat.insert(flat.end(), nodes.begin(), nodes.end());
    if (fast_kind(fast)) {
      // The fast paths' def-side ports: the root's two, then the switch's CON's two.
      const Pair root = nodes[fast_field(fast, 0)];
      flat.push_back(root);
      flat.push_back(fast_kind(fast) == FAST_SWITCH ? nodes[fast_field(fast, 2)] : root);
    }
    if (h.node_len > max_nodes) max_nodes = h.node_len;
    if (vars_len > max_vars) max_vars = vars_len;
  }
  if (flat.empty()) flat.push_back(0);
}

// FNV-1a over the def tables: identifies the book a compiled program was
// emitted for.
static uint64_t tables_hash(const std::vector<DefHdr>& hdr, const std::vector<Pair>& flat) {
  uint64_t x = 0xCBF29CE484222325ull;
  auto mix = [&](const void* p, size_t n) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < n; i++) { x ^= b[i]; x *= 0x100000001B3ull; }
  };
  mix(hdr.data(), hdr.size() * sizeof(DefHdr));
  mix(flat.data(), flat.size() * sizeof(Pair));
  return x;
}

#ifdef HVM_COMPILED_CALLS
uint64_t compiled_book_hash();  // emitted with the compiled calls
#endif

// Limits of the compiled calls: the code is inlined at the CALL sites of
// every turn kernel variant, so only the defs that run repeatedly are
// compiled, up to these totals.
constexpr size_t COMPILED_MAX_DEFS = 256;
constexpr size_t COMPILED_MAX_WORDS = 8192;  // node words + links

// The defs that lie on a cycle of the book's REF graph (recursive functions)
// and the defs these call: the ones a run calls over and over. A book's data
// defs (called once each, from @main) are not among them.
static std::vector<bool> recursive_defs(const std::vector<HostDef>& defs) {
  const size_t n = defs.size();
  std::vector<std::vector<uint32_t>> out(n);
  for (size_t f = 0; f < n; f++) {
    auto add = [&](Port q) {
      if (get_tag(q) == REF && (get_val(q) & 0xFFFFFFFu) < n) out[f].push_back(get_val(q) & 0xFFFFFFFu);
    };
    add(defs[f].root);
    for (Pair p : defs[f].rbag) { add(get_fst(p)); add(get_snd(p)); }
    for (Pair p : defs[f].node) { add(get_fst(p)); add(get_snd(p)); }
  }
  // Tarjan's strongly connected components, with an explicit stack.
  std::vector<int> index(n, -1), low(n, 0);
  std::vector<bool> on(n, false), rec(n, false);
  std::vector<uint32_t> stack;
  std::vector<std::pair<uint32_t, size_t>> work;  // (def, next edge)
  int next = 0;
  for (uint32_t s = 0; s < n; s++) {
    if (index[s] >= 0) continue;
    work.push_back({s, 0});
    while (!work.empty()) {
      const uint32_t v = work.back().first;
      size_t& k = work.back().second;
      if (k == 0 && index[v] < 0) { index[v] = low[v] = next++; stack.push_back(v); on[v] = true; }
      if (k < out[v].size()) {
        const uint32_t w = out[v][k++];
        if (index[w] < 0) work.push_back({w, 0});
        else if (on[w]) low[v] = std::min(low[v], index[w]);
        continue;
      }
      if (low[v] == index[v]) {
        std::vector<uint32_t> comp;
        uint32_t w;
        do { w = stack.back(); stack.pop_back(); on[w] = false; comp.push_back(w); } while (w != v);
        const bool self = std::find(out[v].begin(), out[v].end(), v) != out[v].end();
        if (comp.size() > 1 || self)
          for (uint32_t c : comp) rec[c] = true;
      }
      work.pop_back();
      if (!work.empty()) low[work.back().first] = std::min(low[work.back().first], low[v]);
    }
  }
  // With everything a recursive def calls (its non-recursive helpers).
  std::vector<uint32_t> todo;
  for (uint32_t f = 0; f < n; f++) if (rec[f]) todo.push_back(f);
  while (!todo.empty()) {
    const uint32_t v = todo.back();
    todo.pop_back();
    for (uint32_t w : out[v]) if (!rec[w]) { rec[w] = true; todo.push_back(w); }
  }
  return rec;
}

// A def name as it may appear in a `//` comment of generated code: the
// front-end's name characters, anything else (a trailing backslash would
// splice the next line into the comment) as '?'.
static std::string comment_name(const std::string& name) {
  std::string r;
  for (char ch : name) {
    const bool ok = (ch >= 'a' && ch <= 'z') || (ch >= 'A' && ch <= 'Z') || (ch >= '0' && ch <= '9') || ch == '_' ||
                    ch == '.' || ch == '-' || ch == '/';
    r += ok ? ch : '?';
  }
  return r;
}

// CUDA source of the compiled calls for a book (see compiled_call_nodes in
// the evaluator): per recursive def, its node stores and its links with the
// fresh node / var bases added to the def-local indices.
static std::string compiled_calls_source(const std::vector<HostDef>& defs) {
  std::vector<DefHdr> hdr;
  std::vector<Pair> flat;
  uint32_t mn = 0, mv = 0;
  def_tables(defs, hdr, flat, mn, mv);
  std::vector<bool> pick = recursive_defs(defs);
  size_t ndefs = 0, words = 0;
  for (size_t f = 0; f < defs.size(); f++) {
    if (!pick[f]) continue;
    const size_t w = hdr[f].node_len + hdr[f].rbag_len;
    if (ndefs + 1 > COMPILED_MAX_DEFS || words + w > COMPILED_MAX_WORDS) { pick[f] = false; continue; }
    ndefs++;
    words += w;
  }
  static const char* tags[8] = {"VAR", "REF", "ERA", "NUM", "CON", "DUP", "OPR", "SWI"};
  auto port = [&](Port q) -> std::string {
    char b[64];
    if (q == CALLER_PORT) return "caller";
    const Tag t = get_tag(q);
    if (t >= CON) snprintf(b, sizeof b, "new_port(%s, nb + %uu)", tags[t], (unsigned)get_val(q));
    else if (t == VAR) snprintf(b, sizeof b, "new_port(VAR, vb + %uu)", (unsigned)get_val(q));
    else snprintf(b, sizeof b, "0x%08xu", (unsigned)q);  // REF/ERA/NUM: below 2^32 in either width
    return b;
  };
  std::string o;
  char line[96];
  o += "\n// ---- compiled calls (hvm gen-cu --compiled) ----\n";
  o += "HVM_NS_BEGIN\n";
  snprintf(line, sizeof line, "// %zu of %zu defs compiled (the recursive ones and their callees)\n", ndefs, defs.size());
  o += line;
  o += "__device__ __forceinline__ bool compiled_call_nodes(const Dev& d, uint32_t fid, uint32_t nb, uint32_t vb) {\n";
  o += "  (void)d; (void)nb; (void)vb;\n";
  o += "  switch (fid) {\n";
  for (size_t f = 0; f < defs.size(); f++) {
    if (!pick[f]) continue;
    o += "    case " + std::to_string(f) + "u:  // " + comment_name(defs[f].name) + "\n";
    const Pair* nodes = flat.data() + hdr[f].off + hdr[f].rbag_len;
    for (uint32_t i = 0; i < hdr[f].node_len; i++) {
      snprintf(line, sizeof line, "      nstore(d, nb + %uu, new_pair(", i);
      o += line + port(get_fst(nodes[i])) + ", " + port(get_snd(nodes[i])) + "));\n";
    }
    o += "      return true;\n";
  }
  o += "    default: return false;\n  }\n}\n\n";
  o += "__device__ __forceinline__ bool compiled_call_link(uint32_t fid, uint32_t i, uint32_t nb, uint32_t vb, Port caller,\n";
  o += "                                                   Port& x, Port& y) {\n";
  o += "  (void)i; (void)nb; (void)vb; (void)caller; (void)x; (void)y;\n";
  o += "  switch (fid) {\n";
  for (size_t f = 0; f < defs.size(); f++) {
    if (!pick[f]) continue;
    o += "    case " + std::to_string(f) + "u:  // " + comment_name(defs[f].name) + "\n      switch (i) {\n";
    const Pair* links = flat.data() + hdr[f].off;
    for (uint32_t i = 0; i < hdr[f].rbag_len; i++) {
      snprintf(line, sizeof line, "        case %uu: x = ", i);
      o += line + port(get_fst(links[i])) + "; y = " + port(get_snd(links[i])) + "; return true;\n";
    }
    o += "        default: return false;\n      }\n";
  }
  o += "    default: return false;\n  }\n}\n\n";
  snprintf(line, sizeof line, "uint64_t compiled_book_hash() { return 0x%016llxull; }\n",
           (unsigned long long)tables_hash(hdr, flat));
  o += line;
  o += "HVM_NS_END\n";
  return o;
}

class Runtime {
 public:
  hvm_gb300_config cfg;
  std::string err;
  std::vector<HostDef> defs;
  Dev d{};
  Ctl* ctl = nullptr;
  uint32_t nroots = 1;                 // nets in the loaded batch (1 for a single book)
  std::vector<uint32_t> net_main;      // fid of each net's @main
  std::vector<uint32_t> template_main; // the loaded nets' mains, once requests refer to them
  std::vector<Port> roots;             // each net's resolved ROOT after run_batch
  void* mem_roots = nullptr;
  uint32_t roots_cap = 0;
  void* mem_mains = nullptr;
  uint32_t mains_cap = 0;
  void* mem_node = nullptr; void* mem_vars = nullptr; void* mem_ring = nullptr;
  void* mem_cur = nullptr; void* mem_scratch = nullptr;
  void* mem_defs = nullptr; void* mem_book = nullptr; void* mem_trace = nullptr; void* mem_free = nullptr;
  Port* g_out = nullptr; uint32_t* g_kids = nullptr; uint32_t* g_info = nullptr;
  uint32_t gather_cap = 0;
  uint32_t grid = 0, block = 0, cap = 0;
  void (*turn_fn)(Dev, uint32_t) = nullptr;
  // Turn kernel variants: 0 = `reg_cap_blocks`, 1 = `narrow_reg_cap` (used
  // while few redexes are pending, when `narrow_below` is set). Per-thread
  // allocator state and CALL scratch are sized for the larger grid.
  struct Variant {
    void (*fn)(Dev, uint32_t) = nullptr;
    // Persistent form (cfg.persistent): same register cap, cooperative launch.
    void (*pfn)(Dev, uint32_t, uint32_t, unsigned long long, unsigned long long) = nullptr;
    uint32_t grid = 0, nthreads = 0;
  };
  Variant variants[2];
  int cur_variant = 0;
  uint32_t nthreads_max = 0;
  size_t smem = 0;
  uint32_t max_def_nodes = 1, max_def_vars = 1;
  size_t defs_bytes = 0, book_bytes = 0, scratch_bytes = 0;  // capacities of mem_defs / mem_book / mem_scratch
  std::string result_cache;            // the last run's `Result:` text (hvm_gb300_result)
  bool result_valid = false;
  int sms = 0;
  // Host injection region per space (0 = nodes, 1 = vars): [lo, hi) words, next candidate.
  uint32_t host_lo[2] = {0, 0}, host_hi[2] = {0, 0}, host_next[2] = {0, 0};
  // Pools' high-water marks (pages handed out) since the last clear, and
  // whether they were read after the last turn ran (else clear everything).
  uint64_t used_node_pages = 0, used_var_pages = 0;
  bool marks_valid = false;
  uint32_t* list_buf = nullptr;          // device list readback: LIST_READ_MAX values + info
  uint32_t max_pages = MAX_PAGES;        // page-list capacity per thread and space
  // Scheduler policy written into the control block at every reset.
  uint32_t policy_mode = POLICY_FIXED;
  float policy_const[6] = {-1.f, -1.f, -1.f, -1.f, -1.f, -1.f};
  float* mem_policy = nullptr;
  float* mem_script = nullptr;          // POLICY_SCRIPT decisions, 3 floats per turn
  void* mem_ovf = nullptr;              // local-net variant: per-thread overflow stacks
  size_t script_cap = 0, script_len = 0;
  double norm_seconds = 0;
  uint64_t norm_calls = 0;
  // Measurement: device time of turn kernels (events around each launch),
  // launches of this library's kernels, and bytes copied each way.
  std::vector<cudaEvent_t> events;
  uint32_t timed_units = 0;             // event pairs recorded by the last launch_turns
  // CUDA graph of `cfg.graph_turns` turn launches and the Dev it was captured with.
  cudaGraphExec_t gexec = nullptr;
  cudaStream_t cap_stream = nullptr;
  Dev gdev{};
  double kernel_ms = 0;
  uint64_t turn_launches = 0, launches = 0, h2d_bytes = 0, d2h_bytes = 0;

  ~Runtime() {
    for (cudaEvent_t e : events) cudaEventDestroy(e);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (cap_stream) cudaStreamDestroy(cap_stream);
    release();
  }

  void count_reset() { kernel_ms = 0; turn_launches = launches = h2d_bytes = d2h_bytes = 0; }

  int fail(const std::string& m) { if (err.empty()) err = m; return -1; }

  void release() {
    void* ps[] = {mem_node, mem_vars, mem_ring, mem_cur, mem_scratch, mem_defs, mem_book, g_out, g_kids, g_info, ctl,
                  mem_trace, mem_roots, mem_free, mem_mains, mem_policy, mem_script, mem_ovf, list_buf};
    for (void* p : ps) if (p) cudaFree(p);
    mem_node = mem_vars = mem_ring = mem_cur = mem_scratch = mem_defs = mem_book = mem_trace = mem_roots = mem_free =
        mem_mains = nullptr;
    mem_policy = nullptr;
    mem_script = nullptr;
    mem_ovf = nullptr;
    script_cap = script_len = 0;
    list_buf = nullptr;
    defs_bytes = book_bytes = scratch_bytes = 0;
    g_out = nullptr; g_kids = nullptr; g_info = nullptr; ctl = nullptr;
  }

  int init(const hvm_gb300_config* c) {
    hvm_gb300_default_config(&cfg);
    if (c) cfg = *c;
    CK(cudaSetDevice(cfg.device));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device));
    block = cfg.threads_per_block;
    cap = cfg.stack_cap;
    if (block == 0 || block % 32 || block > 128) return fail("threads_per_block must be a multiple of 32 in [32, 128]");
    if (cap < 2 || (cap & (cap - 1))) return fail("stack_cap must be a power of two >= 2");
    // Word indices are 32-bit; 32-bit ports address 2^29 words.
    const uint32_t max_log2 = PORT_BITS == 64 ? 32 : 29;
    if (cfg.node_log2 < 10 || cfg.node_log2 > max_log2 || cfg.vars_log2 < 10 || cfg.vars_log2 > max_log2)
      return fail(PORT_BITS == 64 ? "node_log2/vars_log2 must be in [10, 32]" : "node_log2/vars_log2 must be in [10, 29]");
    if (cfg.upper_half > 1) return fail("upper_half must be 0 or 1");
    smem = (size_t)block * cap * sizeof(Pair);
    if (block > 128) return fail("threads_per_block must be <= 128");
    if (cfg.local_nets > 1) return fail("local_nets must be 0 or 1");
    if (cfg.persistent > 1) return fail("persistent must be 0 or 1");
    if (cfg.persistent && cfg.graph_turns) return fail("persistent and graph_turns are exclusive");
    if (cfg.local_nets) {
      // The block's local net (LOCAL_WORDS nodes and vars: a slice per lane) follows the deques.
      if (block * LOCAL_SLICE != LOCAL_WORDS) return fail("local_nets needs 128-thread blocks");
      smem += (size_t)LOCAL_WORDS * (sizeof(Pair) + sizeof(Port)) + (size_t)block * sizeof(uint32_t);
    }
    // The turn kernel variant (register cap) and its grid; with `narrow_below`,
    // a second variant runs the turns that start with fewer pending redexes.
    auto make_variant = [&](uint32_t reg_cap, Variant& v) -> int {
      // The fast-path, profiling and local-net variants exist for the caps the defaults use.
      const bool fast = cfg.fast_calls != 0, prof = cfg.profile != 0, local = cfg.local_nets != 0;
      if ((fast ? 1 : 0) + (prof ? 1 : 0) + (local ? 1 : 0) > 1)
        return fail("fast_calls, profile and local_nets are not compiled together");
      if ((prof || local) && reg_cap != 0 && reg_cap != 8)
        return fail("profile and local_nets need reg_cap_blocks / narrow_reg_cap 0 or 8");
      if (fast && reg_cap == 6) return fail("fast_calls needs reg_cap_blocks / narrow_reg_cap 0, 5 or 8");
#ifdef HVM_PORT64
      // The 64-bit port build compiles the default variants only.
      if (fast || prof || local) return fail("fast_calls, profile and local_nets are not in the 64-bit port build");
      switch (reg_cap) {
        case 0: v.fn = turn_kernel<0, false, false, false>; break;
        case 8: v.fn = turn_kernel<8, false, false, false>; break;
        default: return fail("the 64-bit port build has register caps 0 and 8");
      }
#else
      switch (reg_cap) {
        case 0: v.fn = fast ? turn_kernel<0, true, false, false> : prof ? turn_kernel<0, false, true, false>
                     : local ? turn_kernel<0, false, false, true> : turn_kernel<0, false, false, false>; break;
        case 5: v.fn = fast ? turn_kernel<5, true, false, false> : turn_kernel<5, false, false, false>; break;
        case 6: v.fn = turn_kernel<6, false, false, false>; break;
        case 8: v.fn = fast ? turn_kernel<8, true, false, false> : prof ? turn_kernel<8, false, true, false>
                     : local ? turn_kernel<8, false, false, true> : turn_kernel<8, false, false, false>; break;
        default: return fail("reg_cap_blocks / narrow_reg_cap must be 0, 5, 6 or 8");
      }
#endif
      CK(cudaFuncSetAttribute(v.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      int per_sm = 0;
      CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v.fn, (int)block, smem));
      if (cfg.persistent) {
        if (fast || prof || local) return fail("persistent is not compiled with fast_calls, profile or local_nets");
        if (reg_cap == 0) v.pfn = persistent_kernel<0>;
        else if (reg_cap == 8) v.pfn = persistent_kernel<8>;
        else return fail("persistent needs reg_cap_blocks / narrow_reg_cap 0 or 8");
        CK(cudaFuncSetAttribute(v.pfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int p_sm = 0;  // every block of a cooperative launch must be resident
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p_sm, v.pfn, (int)block, smem));
        per_sm = std::min(per_sm, p_sm);
      }
      if (per_sm <= 0) return fail("turn kernel does not fit on an SM with this block size / stack capacity");
      if (cfg.blocks_per_sm && (int)cfg.blocks_per_sm < per_sm) per_sm = (int)cfg.blocks_per_sm;
      v.grid = (uint32_t)(per_sm * sms);
      v.nthreads = v.grid * block;
      return 0;
    };
    if (make_variant(cfg.reg_cap_blocks, variants[0])) return -1;
    variants[1] = variants[0];
    if (cfg.narrow_below && make_variant(cfg.narrow_reg_cap, variants[1])) return -1;
    cur_variant = 0;
    turn_fn = variants[0].fn;
    grid = variants[0].grid;
    uint32_t nthreads = variants[0].nthreads;
    nthreads_max = std::max(variants[0].nthreads, variants[1].nthreads);

    uint64_t n_nodes = 1ull << cfg.node_log2, n_vars = 1ull << cfg.vars_log2;
    d.nthreads = nthreads;
    if (cfg.steal_min == 1 || cfg.steal_min > cap) return fail("steal_min must be 0 or in [2, stack_cap]");
    d.steal_min = cfg.steal_min ? cfg.steal_min : 2;
    if (cfg.rule_select > 2) return fail("rule_select must be 0, 1 or 2");
    d.rule_select = cfg.rule_select;
    if (cfg.fast_calls > 2) return fail("fast_calls must be 0, 1 or 2");
    d.fast_calls = cfg.fast_calls;
    // Pages: a power of two of words, at most 512 node / 1024 var words, and
    // small enough that every thread starts with one page and at least as
    // many pages again remain in the pool.
    auto page_log2_for = [&](uint64_t words, uint32_t max_log2, uint32_t min_log2) -> int {
      int l = (int)max_log2;
      while (l >= (int)min_log2 && (words >> l) < 2ull * nthreads_max) l--;
      return l < (int)min_log2 ? -1 : l;
    };
    if ((cfg.node_page_log2 && (cfg.node_page_log2 < 5 || cfg.node_page_log2 > 12)) ||
        (cfg.var_page_log2 && (cfg.var_page_log2 < 5 || cfg.var_page_log2 > 12)))
      return fail("node_page_log2/var_page_log2 must be 0 or in [5, 12]");
    int nl = page_log2_for(n_nodes, cfg.node_page_log2 ? cfg.node_page_log2 : 9, 5);
    int vl = page_log2_for(n_vars, cfg.var_page_log2 ? cfg.var_page_log2 : 10, 5);
    if (nl < 0 || vl < 0) return fail("node/var space too small for the thread count");
    d.nspace.page_log2 = (uint32_t)nl;
    d.vspace.page_log2 = (uint32_t)vl;
    // Page-list capacity: by default enough for 2^15 node words and 2^16 var
    // words per thread (64 pages of the default sizes), at least 64 pages.
    uint32_t mp = cfg.max_pages;
    if (!mp) {
      uint32_t a = (1u << 15) >> nl, b = (1u << 16) >> vl;
      mp = a > b ? a : b;
      if (mp < MAX_PAGES) mp = MAX_PAGES;
    }
    if (mp > 4096) return fail("max_pages must be at most 4096");
    max_pages = mp;
    d.nspace.max_pages = d.vspace.max_pages = mp;
    d.npool_end = (uint32_t)(n_nodes >> nl);
    d.vpool_end = (uint32_t)(n_vars >> vl);
    d.node_mask = (uint32_t)(n_nodes - 1);
    CK(cudaMalloc(&mem_node, n_nodes * sizeof(Pair)));
    CK(cudaMalloc(&mem_vars, n_vars * sizeof(Port)));
    d.vars_mask = (uint32_t)(n_vars - 1);
    uint64_t ring_len = 1ull << cfg.ring_log2;
    CK(cudaMalloc(&mem_ring, ring_len * sizeof(Pair)));
    // Page lists + counts + positions + offsets, for both spaces.
    CK(cudaMalloc(&mem_cur, 2ull * nthreads_max * (max_pages + 3) * sizeof(uint32_t)));
    CK(cudaMalloc((void**)&ctl, sizeof(Ctl)));
    d.ovf = nullptr;
    if (cfg.local_nets) {
      CK(cudaMalloc((void**)&mem_ovf, (size_t)nthreads_max * OVF_CAP * sizeof(Pair)));
      d.ovf = (Pair*)mem_ovf;
    }
    {
      // One free-page ring per space, as large as the space's page count.
      uint64_t np = n_nodes >> d.nspace.page_log2, vp = n_vars >> d.vspace.page_log2;
      CK(cudaMalloc(&mem_free, (np + vp) * sizeof(uint32_t)));
      d.nfree_ring = (uint32_t*)mem_free;
      d.vfree_ring = d.nfree_ring + np;
      d.nfree_mask = (uint32_t)(np - 1);
      d.vfree_mask = (uint32_t)(vp - 1);
    }
    d.node = (Pair*)mem_node;
    d.vars = (Port*)mem_vars;
    d.ring = (Pair*)mem_ring;
    d.ring_mask = ring_len - 1;
    uint32_t* w = (uint32_t*)mem_cur;
    for (PagedSpace* sp : {&d.nspace, &d.vspace}) {
      sp->lists = w; w += (size_t)nthreads_max * max_pages;
      sp->counts = w; w += nthreads_max;
      sp->pos = w; w += nthreads_max;
      sp->off = w; w += nthreads_max;
    }
    d.ctl = ctl;
    return reset_net();
  }

  // Clears the whole net (node/var words, ring, cursors, counters).
  // Clears the net for the next evaluation. Device code writes net words
  // only in pages the allocator handed out -- below the pools' high-water
  // marks, which every control-block read records -- and in the host region
  // and ROOT vars above the pools' ends; so after a run whose marks were
  // read, only those words are cleared, and the whole space otherwise.
  int clear_net() {
    const uint64_t n_nodes = 1ull << cfg.node_log2, n_vars = 1ull << cfg.vars_log2;
    if (!marks_valid) {
      CK(cudaMemset(mem_node, 0, n_nodes * sizeof(Pair)));
      CK(cudaMemset(mem_vars, 0, n_vars * sizeof(Port)));
    } else {
      const uint64_t nlo = std::min<uint64_t>(used_node_pages, d.npool_end) << d.nspace.page_log2;
      const uint64_t vlo = std::min<uint64_t>(used_var_pages, d.vpool_end) << d.vspace.page_log2;
      const uint64_t ntop = (uint64_t)d.npool_end << d.nspace.page_log2;
      const uint64_t vtop = (uint64_t)d.vpool_end << d.vspace.page_log2;
      CK(cudaMemset(mem_node, 0, nlo * sizeof(Pair)));
      CK(cudaMemset(mem_vars, 0, vlo * sizeof(Port)));
      CK(cudaMemset((Pair*)mem_node + ntop, 0, (n_nodes - ntop) * sizeof(Pair)));
      CK(cudaMemset((Port*)mem_vars + vtop, 0, (n_vars - vtop) * sizeof(Port)));
    }
    marks_valid = false;
    used_node_pages = used_var_pages = 0;
    return 0;
  }

  int reset_net() {
    result_valid = false;
    if (clear_net()) return -1;
    // The top `nroots` var words are ROOT vars: no page that holds one is handed out.
    d.vpool_end = (uint32_t)(((1ull << cfg.vars_log2) - nroots) >> d.vspace.page_log2);
    // The last pages below each pool's end are the host's: IO results are
    // written there (host_take), never by the device allocator.
    {
      const uint64_t hn_words = std::min<uint64_t>(HOST_NODE_WORDS, (1ull << cfg.node_log2) / 64);
      const uint64_t hv_words = std::min<uint64_t>(HOST_VAR_WORDS, (1ull << cfg.vars_log2) / 64);
      const uint32_t hn = std::max<uint32_t>(1u, (uint32_t)(hn_words >> d.nspace.page_log2));
      const uint32_t hv = std::max<uint32_t>(1u, (uint32_t)(hv_words >> d.vspace.page_log2));
      const uint32_t nfull = (uint32_t)((1ull << cfg.node_log2) >> d.nspace.page_log2);
      if (nfull <= nthreads_max + hn + reserved_pages(d.nspace.page_log2) ||
          d.vpool_end <= nthreads_max + hv + reserved_pages(d.vspace.page_log2))
        return fail("node/var space too small for the thread count");
      d.npool_end = nfull - hn;
      d.vpool_end -= hv;
      // upper_half: the pools start at the middle of each space.
      d.npool_base = reserved_pages(d.nspace.page_log2) + (cfg.upper_half ? d.npool_end / 2 : 0);
      d.vpool_base = reserved_pages(d.vspace.page_log2) + (cfg.upper_half ? d.vpool_end / 2 : 0);
      if (d.npool_base + nthreads_max >= d.npool_end || d.vpool_base + nthreads_max >= d.vpool_end)
        return fail("node/var space too small for the thread count");
      host_lo[0] = d.npool_end << d.nspace.page_log2;
      host_hi[0] = (uint32_t)std::min<uint64_t>((uint64_t)(d.npool_end + hn) << d.nspace.page_log2, d.node_mask);
      host_lo[1] = d.vpool_end << d.vspace.page_log2;
      host_hi[1] = (d.vpool_end + hv) << d.vspace.page_log2;
      host_next[0] = host_lo[0];
      host_next[1] = host_lo[1];
    }
    if (d.vpool_end < nthreads_max) return fail("var space too small for this batch");
    CK(cudaMemset(ctl, 0, sizeof(Ctl)));
    if (cfg.profile) { uint32_t one = 1; CK(cudaMemcpy(&ctl->prof_on, &one, sizeof(one), cudaMemcpyHostToDevice)); }
    uint32_t frac = cfg.stop_frac_q8 ? cfg.stop_frac_q8 : 32;
    CK(cudaMemcpy(&ctl->stop_frac_q8, &frac, sizeof(frac), cudaMemcpyHostToDevice));
    if (write_policy()) return -1;
    if (cfg.trace_cap) {
      if (!mem_trace) CK(cudaMalloc(&mem_trace, (size_t)cfg.trace_cap * sizeof(TurnRecord)));
      TurnRecord* tp = (TurnRecord*)mem_trace;
      unsigned cap_ = cfg.trace_cap;
      CK(cudaMemcpy(&ctl->trace, &tp, sizeof(tp), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(&ctl->trace_cap, &cap_, sizeof(cap_), cudaMemcpyHostToDevice));
    }
    // Thread g starts with page g of each space; the pools start after them.
    // Every thread of the larger variant's grid gets its pages.
    {
      Dev all = d;
      all.nthreads = nthreads_max;
      reset_alloc_kernel<<<(nthreads_max + 255) / 256, 256>>>(all);
    }
    CK(cudaGetLastError());
    launches++;
    norm_seconds = 0;
    norm_calls = 0;
    return 0;
  }

  int write_policy() {
    const float* w = policy_mode == POLICY_LEARNED ? mem_policy : policy_mode == POLICY_SCRIPT ? mem_script : nullptr;
    const unsigned sl = policy_mode == POLICY_SCRIPT ? (unsigned)script_len : 0u;
    CK(cudaMemcpy(&ctl->policy_script_len, &sl, sizeof(sl), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(&ctl->policy_mode, &policy_mode, sizeof(policy_mode), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(&ctl->policy_const, policy_const, sizeof(policy_const), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(&ctl->policy_w, &w, sizeof(w), cudaMemcpyHostToDevice));
    const uint32_t bc = cfg.turn_budget_cap;
    CK(cudaMemcpy(&ctl->budget_cap, &bc, sizeof(bc), cudaMemcpyHostToDevice));
    return 0;
  }

  int set_policy(uint32_t mode, const float* weights, size_t n, const float* constants) {
    if (mode > POLICY_SCRIPT) return fail("unknown policy mode");
    if (mode == POLICY_SCRIPT) {
      if ((!weights && n) || n % 3 || n / 3 > (1u << 20)) return fail("a policy script is 3 floats per turn");
      if (n > script_cap) {
        if (mem_script) cudaFree(mem_script);
        mem_script = nullptr;
        script_cap = 0;
        CK(cudaMalloc((void**)&mem_script, n * sizeof(float)));
        script_cap = n;
      }
      if (n) CK(cudaMemcpy(mem_script, weights, n * sizeof(float), cudaMemcpyHostToDevice));
      script_len = n / 3;
    }
    if (mode == POLICY_LEARNED) {
      if (!weights || n != (size_t)POLICY_PARAMS) return fail("learned policy needs HVM_GB300_POLICY_PARAMS weights");
      for (size_t i = 0; i < n; i++)
        if (!std::isfinite(weights[i])) return fail("policy weights must be finite");
      if (!mem_policy) CK(cudaMalloc((void**)&mem_policy, POLICY_PARAMS * sizeof(float)));
      CK(cudaMemcpy(mem_policy, weights, POLICY_PARAMS * sizeof(float), cudaMemcpyHostToDevice));
    }
    if (mode == POLICY_CONSTANT) {
      if (!constants) return fail("constant policy needs 6 constants");
      for (int i = 0; i < 6; i++) policy_const[i] = constants[i];
    }
    policy_mode = mode;
    return write_policy();
  }

  // Parses the book buffer (src/hvm.c:1408-1453 limits and messages).
  int load_book(const uint32_t* w, size_t words) {
    std::vector<HostDef> parsed;
    if (parse_book(w, words, parsed)) return -1;
    defs = std::move(parsed);
    nroots = 1;
    return upload_book();
  }

  // Loads `n` independent nets as one batch: their books are concatenated,
  // with each net's fids (and the REFs that name them) shifted past the
  // previous nets' defs. Net k's `@main` becomes fid net_main[k].
  int load_batch(const uint32_t* const* books, const size_t* words, uint32_t n) {
    if (n == 0) return fail("empty batch");
    if (n > MAX_BATCH) return fail("batch larger than " + std::to_string(MAX_BATCH) + " nets");
    std::vector<HostDef> all;
    std::vector<uint32_t> mains(n);
    for (uint32_t k = 0; k < n; k++) {
      std::vector<HostDef> one;
      if (parse_book(books[k], words ? words[k] : 0, one)) {
        err = "net " + std::to_string(k) + ": " + err;
        return -1;
      }
      uint32_t shift = (uint32_t)all.size();
      if ((uint64_t)shift + one.size() > MAX_BATCH_DEFS) return fail("batch has too many definitions");
      auto remap = [&](Port p) {
        if (get_tag(p) != REF) return p;
        Val v = get_val(p);
        return new_port(REF, (v & 0x10000000u) | ((v & 0xFFFFFFFu) + shift));
      };
      for (HostDef& h : one) {
        h.root = remap(h.root);
        for (Pair& q : h.rbag) q = new_pair(remap(get_fst(q)), remap(get_snd(q)));
        for (Pair& q : h.node) q = new_pair(remap(get_fst(q)), remap(get_snd(q)));
        all.push_back(std::move(h));
      }
      mains[k] = shift;
    }
    defs = std::move(all);
    nroots = n;
    net_main = mains;
    template_main.clear();
    return upload_book();
  }

  // Serving: `n` requests, request r being a copy of loaded net tmpl[r]. The
  // copies share that net's definitions (defs are read-only templates) and
  // each gets its own ROOT var, so nets of the batch become request templates.
  int set_requests(const uint32_t* tmpl, uint32_t n) {
    if (net_main.empty()) return fail("no batch loaded");
    if (n == 0 || n > MAX_BATCH) return fail("request count out of range");
    if (template_main.empty()) template_main = net_main;
    std::vector<uint32_t> mains(n);
    for (uint32_t r = 0; r < n; r++) {
      if (tmpl[r] >= template_main.size()) return fail("request template out of range");
      mains[r] = template_main[tmpl[r]];
    }
    net_main = mains;
    nroots = n;
    return 0;
  }

  int parse_book(const uint32_t* w, size_t words, std::vector<HostDef>& defs) {
    defs.clear();
    if (!w) return fail("null book buffer");
    size_t at = 0;
    auto need = [&](size_t k) { return words == 0 || at + k <= words; };
    if (!need(1)) return fail("failed to load book");
    uint32_t ndefs = w[at++];
    if (ndefs == 0 || ndefs > MAX_DEFS) return fail("failed to load book");
    defs.resize(ndefs);
    std::vector<bool> seen(ndefs, false);
    for (uint32_t k = 0; k < ndefs; k++) {
      if (!need(DEF_HEADER_WORDS)) return fail("failed to load book");
      uint32_t fid = w[at++];
      if (fid >= ndefs) return fail("failed to load book");
      HostDef& h = defs[fid];
      char name[257];
      memcpy(name, &w[at], 256);
      name[256] = 0;
      h.name = name;
      at += 64;
      h.safe = w[at++] != 0;
      h.rbag_len = w[at++];
      h.node_len = w[at++];
      h.vars_len = w[at++];
      if (h.rbag_len > DEF_RBAG_LEN) return fail("def '" + h.name + "' has too many redexes: " + std::to_string(h.rbag_len));
      if (h.node_len > DEF_NODE_LEN) return fail("def '" + h.name + "' has too many nodes: " + std::to_string(h.node_len));
      h.root = w[at++];
      if (!need(2ull * (h.rbag_len + h.node_len))) return fail("failed to load book");
      h.rbag.resize(h.rbag_len);
      h.node.resize(h.node_len);
      for (uint32_t i = 0; i < h.rbag_len; i++, at += 2) h.rbag[i] = new_pair(w[at], w[at + 1]);
      for (uint32_t i = 0; i < h.node_len; i++, at += 2) h.node[i] = new_pair(w[at], w[at + 1]);
      seen[fid] = true;
    }
    // Every def-local port must point inside its def and every REF at a def
    // of this book, so that the device never indexes past its arrays. The
    // reference does not check; a book from the front-end always passes.
    for (uint32_t f = 0; f < ndefs; f++) {
      if (!seen[f]) return fail("failed to load book: missing definition " + std::to_string(f));
      const HostDef& h = defs[f];
      auto ok = [&](Port p) {
        Tag t = get_tag(p);
        if (t >= CON) return get_val(p) < h.node_len;
        if (t == VAR) return get_val(p) < h.vars_len;
        if (t == REF) return (get_val(p) & 0xFFFFFFFu) < ndefs;
        return true;
      };
      bool good = ok(h.root);
      for (Pair p : h.rbag) good = good && ok(get_fst(p)) && ok(get_snd(p));
      for (Pair p : h.node) good = good && ok(get_fst(p)) && ok(get_snd(p));
      if (!good) return fail("failed to load book: def '" + h.name + "' has a port outside the def");
    }
    return 0;
  }

  int upload_book() {
    std::vector<DefHdr> hdr;
    std::vector<Pair> flat;
    def_tables(defs, hdr, flat, max_def_nodes, max_def_vars);
#ifdef HVM_COMPILED_CALLS
    // A program with compiled calls evaluates the book it was emitted for.
    if (tables_hash(hdr, flat) != compiled_book_hash())
      return fail("this program's compiled calls were emitted for another book");
    d.compiled = 1;
#endif
    // Device buffers are kept between loads and grown only when a book needs
    // more (cudaFree synchronises the device; a reload should not).
    auto ensure = [&](void*& p, size_t& have, size_t need) -> int {
      if (p && have >= need) return 0;
      if (p) cudaFree(p);
      p = nullptr;
      have = 0;
      CK(cudaMalloc(&p, need));
      have = need;
      return 0;
    };
    // Relocation tables: for defs larger than a chunk, and as the fallback
    // when a CALL finds no contiguous run; so at least CHUNK words each.
    if (max_def_nodes < CHUNK) max_def_nodes = CHUNK;
    if (max_def_vars < CHUNK) max_def_vars = CHUNK;
    if (ensure(mem_defs, defs_bytes, hdr.size() * sizeof(DefHdr)) ||
        ensure(mem_book, book_bytes, flat.size() * sizeof(Pair)) ||
        ensure(mem_scratch, scratch_bytes, (size_t)(max_def_nodes + max_def_vars) * nthreads_max * sizeof(uint32_t)))
      return -1;
    CK(cudaMemcpy(mem_defs, hdr.data(), hdr.size() * sizeof(DefHdr), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(mem_book, flat.data(), flat.size() * sizeof(Pair), cudaMemcpyHostToDevice));
    h2d_bytes += hdr.size() * sizeof(DefHdr) + flat.size() * sizeof(Pair);
    d.tables = 1;
    d.defs = (const DefHdr*)mem_defs;
    d.book = (const Pair*)mem_book;
    d.ndefs = (uint32_t)defs.size();
    d.nloc = (uint32_t*)mem_scratch;
    d.vloc = d.nloc + (size_t)max_def_nodes * nthreads_max;
    return 0;
  }

  // Makes variant v the one that runs the next turns (between turns, with
  // the device idle) and re-plans the pending turn for its grid.
  int use_variant(int v) {
    if (v == cur_variant) return 0;
    cur_variant = v;
    turn_fn = variants[v].fn;
    grid = variants[v].grid;
    d.nthreads = variants[v].nthreads;
    retarget_kernel<<<1, 1>>>(d, cap);
    CK(cudaGetLastError());
    launches++;
    return 0;
  }

  // After a poll: the narrow variant while fewer than `narrow_below`
  // redexes are pending, else the configured one.
  int pick_variant(const Ctl& h) {
    if (!cfg.narrow_below || h.base == h.in_end) return 0;
    return use_variant(h.in_end - h.base < cfg.narrow_below ? 1 : 0);
  }

  int read_ctl(Ctl& h) {
    CK(cudaMemcpy(&h, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
    d2h_bytes += sizeof(Ctl);
    used_node_pages = std::max(used_node_pages, (uint64_t)h.npool_next);
    used_var_pages = std::max(used_var_pages, (uint64_t)h.vpool_next);
    marks_valid = true;
    return 0;
  }

  // Pushes `redex` and resets `root` (the reference's boot_redex,
  // src/hvm.c:1480-1486, which always resets ROOT).
  int boot_root(Pair redex, Port root) {
    boot_kernel<<<1, 1>>>(d, redex, root, cap);
    CK(cudaGetLastError());
    launches++;
    return 0;
  }

  int boot(Pair redex) {
    boot_kernel<<<1, 1>>>(d, redex, get_snd(redex), cap);
    CK(cudaGetLastError());
    launches++;
    return 0;
  }

  // Captures `cfg.graph_turns` turn launches into a CUDA graph for the
  // current kernel arguments (the Dev block is passed by value, so a changed
  // book or batch means a new capture).
  int ensure_graph() {
    if (gexec && memcmp(&gdev, &d, sizeof(Dev)) == 0) return 0;
    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
    if (!cap_stream) CK(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
    CK(cudaStreamBeginCapture(cap_stream, cudaStreamCaptureModeThreadLocal));
    for (uint32_t i = 0; i < cfg.graph_turns; i++) turn_fn<<<grid, block, smem, cap_stream>>>(d, cap);
    cudaGraph_t gr = nullptr;
    CK(cudaStreamEndCapture(cap_stream, &gr));
    cudaError_t e = cudaGraphInstantiate(&gexec, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) { gexec = nullptr; return fail(std::string("graph instantiation: ") + cudaGetErrorString(e)); }
    memcpy(&gdev, &d, sizeof(Dev));
    return 0;
  }

  // Launches at least n turns on the default stream: single launches, or
  // replays of the captured graph of `cfg.graph_turns` launches. Each launch
  // or replay is bracketed by an event pair that collect_times() reads once
  // the host has synchronised.
  int launch_turns(uint32_t n) {
    const uint32_t g = cfg.graph_turns;
    const uint32_t units = g ? (n + g - 1) / g : n;
    while (events.size() < 2 * (size_t)units) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      events.push_back(e);
    }
    if (g && ensure_graph()) return -1;
    marks_valid = false;  // until the control block is read after these turns
    for (uint32_t i = 0; i < units; i++) {
      CK(cudaEventRecord(events[2 * i]));
      if (g) CK(cudaGraphLaunch(gexec, 0));
      else turn_fn<<<grid, block, smem>>>(d, cap);
      CK(cudaEventRecord(events[2 * i + 1]));
    }
    CK(cudaGetLastError());
    const uint32_t k = g ? units * g : n;
    turn_launches += k;
    launches += k;
    timed_units = units;
    return 0;
  }

  // One cooperative launch of the current variant's persistent kernel: up
  // to `turns` turns, ending early at the normal form, on a failure, or once
  // the pending count leaves the variant's range (narrow_below).
  int launch_persistent(uint32_t turns) {
    unsigned long long lo = 0, hi = ~0ull;
    if (cfg.narrow_below) {
      if (cur_variant == 0) lo = cfg.narrow_below;
      else hi = cfg.narrow_below;
    }
    if (events.size() < 2) {
      for (int i = 0; i < 2; i++) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        events.push_back(e);
      }
    }
    marks_valid = false;
    auto fn = variants[cur_variant].pfn;
    void* args[] = {&d, &cap, &turns, &lo, &hi};
    CK(cudaEventRecord(events[0]));
    CK(cudaLaunchCooperativeKernel((const void*)fn, dim3(grid), dim3(block), args, smem, 0));
    CK(cudaEventRecord(events[1]));
    turn_launches++;
    launches++;
    timed_units = 1;
    return 0;
  }

  int collect_times() {
    for (uint32_t i = 0; i < timed_units; i++) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, events[2 * i], events[2 * i + 1]));
      kernel_ms += ms;
    }
    timed_units = 0;
    return 0;
  }

  // The message of a failed turn, with the allocator's state on out-of-memory.
  std::string device_error(const Ctl& h) const {
    std::string m = std::string("device error: ") + status_text(h.status) + " (info " + std::to_string(h.err_info) + ")";
    if (h.oom_space)
      m += " [" + std::string(h.oom_space == 2 ? "var" : "node") + " pages owned " + std::to_string(h.oom_pages) +
           ", dry chunks " + std::to_string(h.oom_dry) + ", pool " + (h.oom_pool_dry ? "empty" : "not empty") +
           ", pools at " + std::to_string(h.npool_next) + "/" + std::to_string(d.npool_end) + " and " +
           std::to_string(h.vpool_next) + "/" + std::to_string(d.vpool_end) + ", live words " +
           std::to_string(h.live_nodes) + " and " + std::to_string(h.live_vars) + "]";
    return m;
  }

  // Runs turns until the ring is empty (src/hvm.cu:1810-1839).
  int normalize() {
    result_valid = false;  // the net changes
    auto t0 = std::chrono::steady_clock::now();
    uint32_t batch = 4;
    uint64_t turns_run = 0, stalled_turns = 0;
    unsigned long long last_itrs = ~0ull, last_pending = ~0ull;
    Ctl h;
    for (;;) {
      if (cfg.persistent) {
        // A launch runs one turn past the budget, as a poll batch may, so
        // that an exhausted budget is seen below.
        uint64_t k = PERSIST_TURNS;
        if (cfg.max_turns) k = std::min<uint64_t>(k, cfg.max_turns - std::min<uint64_t>(turns_run, cfg.max_turns) + 1);
        if (launch_persistent((uint32_t)k)) return -1;
      } else {
        if (launch_turns(batch)) return -1;
        turns_run += batch;
      }
      if (read_ctl(h) || collect_times()) return -1;
      if (cfg.persistent) turns_run += h.persist_ran;
      if (h.status) return fail(device_error(h));
      if (h.base == h.in_end) break;
      if (cfg.max_turns && turns_run >= cfg.max_turns) return fail("turn budget exhausted before normal form");
      // A net whose interaction count stops moving while redexes remain is
      // stuck (e.g. a redex that never becomes available): report it.
      if (h.itrs == last_itrs && h.pending == last_pending) {
        if (++stalled_turns > (cfg.persistent ? 1u : 4096u))
          return fail("no progress: interaction count stalled with redexes pending");
      } else {
        stalled_turns = 0;
      }
      last_itrs = h.itrs;
      last_pending = h.pending;
      if (pick_variant(h)) return -1;
      if (batch < 64) batch *= 2;
    }
    norm_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    norm_calls++;
    return 0;
  }

  // Single-word device accessors for the host-side readback walk.
  Port vars_load(uint32_t i) {
    Port v = 0;
    cudaMemcpy(&v, d.vars + (i & d.vars_mask), sizeof(Port), cudaMemcpyDeviceToHost);
    d2h_bytes += sizeof(Port);
    return v;
  }
  void vars_store(uint32_t i, Port v) {
    cudaMemcpy(d.vars + (i & d.vars_mask), &v, sizeof(Port), cudaMemcpyHostToDevice);
    h2d_bytes += sizeof(Port);
  }
  Pair node_load(uint32_t i) {
    Pair v = 0;
    cudaMemcpy(&v, d.node + i, sizeof(Pair), cudaMemcpyDeviceToHost);
    d2h_bytes += sizeof(Pair);
    return v;
  }

  // Read-only chase (src/hvm.c:781-790).
  Port peek(Port p) {
    while (get_tag(p) == VAR) {
      Port v = vars_load(get_val(p));
      if (v == NONE || v == 0) break;
      p = v;
    }
    return p;
  }

  // Normalises every REF met by the readback (src/hvm.c:1233-1243). `root`
  // is the net's ROOT var (ROOT, or ROOT_VAR - k for net k of a batch).
  int expand(Port p, Port* out, Port root = ROOT) {
    const uint32_t rv = get_val(root);
    Port saved = vars_load(rv);
    Port got = peek(p);
    while (get_tag(got) == REF) {
      if (boot(new_pair(got, root)) || normalize()) return -1;
      got = peek(vars_load(rv));
    }
    vars_store(rv, saved);
    *out = got;
    return 0;
  }

  struct Ctr { uint32_t tag; uint32_t nargs; Port args[16]; };

  // Lambda-encoded constructor readback (src/run.c:65-97).
  int read_ctr(Port p, Ctr& c, Port root = ROOT) {
    c.tag = (uint32_t)-1;
    c.nargs = 0;
    Port lam, app, arg;
    if (expand(p, &lam, root)) return -1;
    if (get_tag(lam) != CON) return 0;
    Pair lam_n = node_load(get_val(lam));
    if (expand(get_fst(lam_n), &app, root)) return -1;
    if (get_tag(app) != CON) return 0;
    Pair app_n = node_load(get_val(app));
    if (expand(get_fst(app_n), &arg, root)) return -1;
    if (get_tag(arg) != NUM) return 0;
    c.tag = get_u24(get_val(arg));
    for (;;) {
      if (expand(get_snd(app_n), &app, root)) return -1;
      if (get_tag(app) != CON) break;
      app_n = node_load(get_val(app));
      if (expand(get_fst(app_n), &arg, root)) return -1;
      if (c.nargs < 16) c.args[c.nargs] = arg;
      c.nargs++;
    }
    return 0;
  }

  // Every net of a batch: boot @main_k ~ ROOT_k, normalise them together,
  // then run each net's readback walk (which re-normalises REFs it meets).
  int run_batch() {
    if (defs.empty() || nroots < 1 || net_main.size() != nroots) return fail("no batch loaded");
    if (reset_net()) return -1;
    d.extra_roots = nroots - 1;
    uint32_t* dm = nullptr;
    CK(cudaMalloc(&dm, nroots * sizeof(uint32_t)));
    CK(cudaMemcpy(dm, net_main.data(), nroots * sizeof(uint32_t), cudaMemcpyHostToDevice));
    h2d_bytes += nroots * sizeof(uint32_t);
    boot_batch_kernel<<<1, 1024>>>(d, dm, nroots, cap);
    cudaError_t e = cudaGetLastError();
    launches++;
    cudaFree(dm);
    CK(e);
    if (normalize()) return -1;
    if (read_roots()) return -1;
    for (uint32_t k = 0; k < nroots; k++) {
      Tag t = get_tag(roots[k]);
      if (t != REF && t != CON) continue;  // the walk stops at once
      Port root = new_port(VAR, ROOT_VAR - k);
      Ctr c;
      if (read_ctr(peek(root), c, root)) return -1;
    }
    return read_roots();
  }

  // Continuous batching over a loaded batch: net k is admitted once the host
  // clock passes arrival[k] (seconds from the start; non-decreasing), while
  // fewer than `max_inflight` nets are in flight and live node and var words
  // stay under `live_frac` of their spaces. Turns run in small batches; after
  // each, the roots of in-flight nets are checked and a net whose ROOT has
  // become a number is complete (done[k] = host seconds, result[k] = port).
  // When every net is admitted and the ring is empty, the rest complete with
  // whatever their ROOT holds, after the readback expansion.
  // `result` receives each net's result port: a number, so it fits 32 bits
  // in either port width.
  int run_stream(const double* arrival, uint32_t max_inflight, double live_frac, double* done, uint32_t* result,
                 uint32_t order = 0) {
    if (defs.empty() || net_main.size() != nroots) return fail("no batch loaded");
    if (reset_net()) return -1;
    d.extra_roots = nroots - 1;
    if (!mem_mains || mains_cap < nroots) {
      if (mem_mains) cudaFree(mem_mains);
      mem_mains = nullptr;
      CK(cudaMalloc(&mem_mains, 3ull * nroots * sizeof(uint32_t)));
      mains_cap = nroots;
    }
    uint32_t* dm = (uint32_t*)mem_mains;
    uint32_t* dact = dm + nroots;        // nets being admitted
    uint32_t* dlive = dm + 2ull * nroots;  // nets in flight
    CK(cudaMemcpy(dm, net_main.data(), nroots * sizeof(uint32_t), cudaMemcpyHostToDevice));
    h2d_bytes += nroots * sizeof(uint32_t);
    if (read_roots_alloc()) return -1;
    const long long node_limit = (long long)(live_frac * (double)(1ull << cfg.node_log2));
    const long long var_limit = (long long)(live_frac * (double)(1ull << cfg.vars_log2));
    std::vector<uint32_t> active;
    std::vector<Port> ports;
    uint32_t next = 0;         // nets [0, next) have arrived and been queued
    // Arrived nets wait in `ready`; order 0 admits them first come, first
    // served; order 1 admits the smallest book first (among those arrived),
    // which starts the light, often long-running nets early in a batch.
    std::vector<uint32_t> ready;
    size_t ready_head = 0;
    uint32_t admitted_total = 0;
    // A net's weight: the size of the def block its @main starts.
    const std::vector<uint32_t>& blocks = template_main.empty() ? net_main : template_main;
    auto book_words = [&](uint32_t net) -> uint64_t {
      uint32_t lo = net_main[net];
      auto it = std::upper_bound(blocks.begin(), blocks.end(), lo);
      uint32_t hi = it == blocks.end() ? (uint32_t)defs.size() : *it;
      uint64_t w = 0;
      for (uint32_t f = lo; f < hi; f++) w += defs[f].node_len + defs[f].rbag_len;
      return w;
    };
    std::vector<uint64_t> weight;
    if (order == 1) {
      weight.resize(nroots);
      for (uint32_t k = 0; k < nroots; k++) weight[k] = book_words(k);
    }
    std::vector<uint32_t> admit;
    uint32_t stream_cap = cfg.turn_budget_cap;  // the cap written at reset
    Ctl h;
    memset(&h, 0, sizeof(h));
    auto t0 = std::chrono::steady_clock::now();
    auto now_s = [&]() { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    uint64_t polls = 0, stalled_polls = 0;
    for (;;) {
      double now = now_s();
      // Arrivals join the ready queue; admission takes from it.
      size_t before = ready.size();
      while (next < nroots && arrival[next] <= now) ready.push_back(next++);
      if (order == 1 && ready.size() > before) {
        std::stable_sort(ready.begin() + ready_head, ready.end(),
                         [&](uint32_t x, uint32_t y) { return weight[x] < weight[y]; });
      }
      admit.clear();
      while (ready_head < ready.size() && active.size() + admit.size() < max_inflight &&
             h.live_nodes < node_limit && h.live_vars < var_limit && admit.size() < 4096)
        admit.push_back(ready[ready_head++]);
      // Progress: with nothing in flight, a waiting net is admitted whatever
      // the counters say (so the stream cannot stop with nets still queued).
      if (admit.empty() && active.empty() && ready_head < ready.size()) admit.push_back(ready[ready_head++]);
      if (!admit.empty()) {
        CK(cudaMemcpy(dact, admit.data(), admit.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
        h2d_bytes += admit.size() * sizeof(uint32_t);
        admit_kernel<<<1, 1024>>>(d, dm, dact, (uint32_t)admit.size(), cap);
        CK(cudaGetLastError());
        launches++;
        for (uint32_t net : admit) active.push_back(net);
        admitted_total += (uint32_t)admit.size();
      }
      // Turns are capped (cfg.turn_budget_cap) only while no admitted-ready
      // request waits: a short turn then bounds the latency of arrivals and
      // completions; with a backlog, longer turns keep the host out of the way.
      {
        const uint32_t want_cap = ready_head < ready.size() ? 0u : cfg.turn_budget_cap;
        if (want_cap != stream_cap) {
          CK(cudaMemcpy(&ctl->budget_cap, &want_cap, sizeof(want_cap), cudaMemcpyHostToDevice));
          h2d_bytes += sizeof(want_cap);
          stream_cap = want_cap;
        }
      }
      // A few turns, then the control block.
      if (launch_turns(4)) return -1;
      if (read_ctl(h) || collect_times()) return -1;
      if (h.status) return fail(device_error(h));
      if (pick_variant(h)) return -1;
      // Completions.
      const size_t active_before = active.size();
      if (!active.empty()) {
        CK(cudaMemcpy(dlive, active.data(), active.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
        active_roots_kernel<<<((uint32_t)active.size() + 255) / 256, 256>>>(d, dlive, (Port*)mem_roots,
                                                                          (uint32_t)active.size());
        CK(cudaGetLastError());
        launches++;
        ports.resize(active.size());
        CK(cudaMemcpy(ports.data(), mem_roots, active.size() * sizeof(Port), cudaMemcpyDeviceToHost));
        h2d_bytes += active.size() * sizeof(uint32_t);
        d2h_bytes += active.size() * sizeof(Port);
        double t = now_s();
        size_t w = 0;
        for (size_t i = 0; i < active.size(); i++) {
          if (get_tag(ports[i]) == NUM) {
            done[active[i]] = t;
            result[active[i]] = (uint32_t)ports[i];
          } else {
            active[w++] = active[i];
          }
        }
        active.resize(w);
      }
      polls++;
      const bool quiet = h.base == h.in_end;
      if (quiet && admitted_total == nroots) break;
      // A quiet ring with nothing admitted, nothing completed and no arrival
      // still to come cannot change: fail instead of polling forever.
      const bool progressed = !admit.empty() || active.size() != active_before;
      const bool arrival_due = next < nroots && arrival[next] > now_s();
      stalled_polls = quiet && !progressed && !arrival_due ? stalled_polls + 1 : 0;
      if (stalled_polls > 64) return fail("stream stalled: the ring is empty and no net completes or can be admitted");
      if (quiet && active.empty() && ready_head == ready.size() && next < nroots && arrival[next] > now_s()) {
        // Idle until the next arrival.
        while (arrival[next] > now_s()) {}
      }
      if (cfg.max_turns && turn_launches >= cfg.max_turns) return fail("turn budget exhausted before normal form");
    }
    // Quiescent: nets whose ROOT is not a number finish with the readback walk.
    for (uint32_t net : active) {
      Port root = new_port(VAR, ROOT_VAR - net);
      Ctr c;
      if (read_ctr(peek(root), c, root)) return -1;
      done[net] = now_s();
      result[net] = peek(root);
    }
    norm_calls++;
    return 0;
  }

  int read_roots_alloc() {
    if (!mem_roots || roots_cap < nroots) {
      if (mem_roots) cudaFree(mem_roots);
      mem_roots = nullptr;
      CK(cudaMalloc(&mem_roots, nroots * sizeof(Port)));
      roots_cap = nroots;
    }
    return 0;
  }

  int read_roots() {
    if (!mem_roots || roots_cap < nroots) {
      if (mem_roots) cudaFree(mem_roots);
      mem_roots = nullptr;
      CK(cudaMalloc(&mem_roots, nroots * sizeof(Port)));
      roots_cap = nroots;
    }
    batch_roots_kernel<<<(nroots + 255) / 256, 256>>>(d, (Port*)mem_roots, nroots);
    CK(cudaGetLastError());
    launches++;
    roots.resize(nroots);
    CK(cudaMemcpy(roots.data(), mem_roots, nroots * sizeof(Port), cudaMemcpyDeviceToHost));
    d2h_bytes += nroots * sizeof(Port);
    return 0;
  }

  // boot @main ~ ROOT, then the IO loop without IO builtins (src/run.cu:857-925).
  // ---- IO (src/run.c:32-810) ---------------------------------------------
  //
  // The program's ROOT is read back as a lambda-encoded IO constructor; an
  // IO_CALL names a host function, its argument and a continuation. The host
  // reads the argument back, runs the function, writes its result into the
  // net (the host injection region, one copy per structure) and boots
  // `(result, ROOT) ~ continuation`, until an IO_DONE (or anything else).

  // A run of n free words of one space in the host region (0 = nodes,
  // 1 = vars): candidates are read back once and must all be 0 (free).
  int host_take(int sp, uint32_t n, uint32_t& base) {
    const uint32_t span = host_hi[sp] - host_lo[sp];
    if (n == 0 || n > span) return fail("IO result larger than the host injection region");
    std::vector<uint64_t> w(n);
    for (uint32_t moved = 0; moved <= 2 * span;) {
      uint32_t at = host_next[sp];
      if (at + n > host_hi[sp]) { moved += host_hi[sp] - at; host_next[sp] = host_lo[sp]; continue; }
      if (sp == 0) CK(cudaMemcpy(w.data(), d.node + at, n * sizeof(Pair), cudaMemcpyDeviceToHost));
      else {
        std::vector<uint32_t> v(n);
        CK(cudaMemcpy(v.data(), d.vars + at, n * sizeof(Port), cudaMemcpyDeviceToHost));
        for (uint32_t i = 0; i < n; i++) w[i] = v[i];
      }
      d2h_bytes += (uint64_t)n * (sp == 0 ? sizeof(Pair) : sizeof(Port));
      uint32_t last = n;
      for (uint32_t i = 0; i < n; i++) if (w[i]) last = i;
      if (last == n) { base = at; host_next[sp] = at + n; return 0; }
      host_next[sp] = at + last + 1;
      moved += last + 1;
    }
    return fail("IO host injection region is full");
  }

  // Builds a small net on the host: nodes and vars numbered locally, written
  // into the host region in one copy each by commit(). A port is either one
  // of the net's own ports (external) or a local node / local var.
  struct LPort {
    Port p;
    uint8_t kind;  // 0 external, 1 local node (CON), 2 local var
  };
  struct Inject {
    std::vector<std::pair<LPort, LPort>> nodes;
    uint32_t nvars = 0;
    LPort var() { return LPort{new_port(VAR, nvars++), 2}; }
    LPort node(LPort a, LPort b) {
      nodes.push_back({a, b});
      return LPort{new_port(CON, (uint32_t)nodes.size() - 1), 1};
    }
  };
  static LPort ext(Port p) { return LPort{p, 0}; }

  // Places an Inject in the host region and returns where `p` landed.
  int commit(Inject& in, LPort p, Port& out) {
    uint32_t nb = 0, vb = 0;
    if (!in.nodes.empty() && host_take(0, (uint32_t)in.nodes.size(), nb)) return -1;
    if (in.nvars && host_take(1, in.nvars, vb)) return -1;
    auto rel = [&](LPort q) -> Port {
      if (q.kind == 1) return new_port(get_tag(q.p), nb + get_val(q.p));
      if (q.kind == 2) return new_port(VAR, vb + get_val(q.p));
      return q.p;
    };
    std::vector<Pair> ns(in.nodes.size());
    for (size_t i = 0; i < ns.size(); i++) ns[i] = new_pair(rel(in.nodes[i].first), rel(in.nodes[i].second));
    if (!ns.empty()) CK(cudaMemcpy(d.node + nb, ns.data(), ns.size() * sizeof(Pair), cudaMemcpyHostToDevice));
    if (in.nvars) {
      std::vector<Port> vs(in.nvars, NONE);
      CK(cudaMemcpy(d.vars + vb, vs.data(), vs.size() * sizeof(Port), cudaMemcpyHostToDevice));
    }
    h2d_bytes += ns.size() * sizeof(Pair) + (uint64_t)in.nvars * sizeof(Port);
    out = rel(p);
    return 0;
  }

  // Lambda-encoded constructor lam t ((((t TAG) a0) a1) ...) (src/run.c:184-374):
  // application nodes (arg, result) from the tag outwards, the innermost
  // result and the lambda's body sharing one var.
  static LPort ctr_in(Inject& in, uint32_t tag, const LPort* args, uint32_t n) {
    LPort r = in.var();
    LPort chain = r;
    for (uint32_t i = n; i-- > 0;) chain = in.node(args[i], chain);
    LPort first = in.node(ext(new_port(NUM, new_u24(tag))), chain);
    return in.node(first, r);
  }

  int inject_bytes(const std::string& b, Port& out) {
    Inject in;
    LPort list = ctr_in(in, LIST_NIL_TAG, nullptr, 0);
    for (size_t i = b.size(); i-- > 0;) {
      LPort args[2] = {ext(new_port(NUM, new_u24((uint32_t)(uint8_t)b[i]))), list};
      list = ctr_in(in, LIST_CONS_TAG, args, 2);
    }
    return commit(in, list, out);
  }
  int inject_ctr(uint32_t tag, Port a, Port& out) {
    Inject in;
    LPort arg = ext(a);
    return commit(in, ctr_in(in, tag, &arg, 1), out);
  }
  int inject_ok(Port v, Port& out) { return inject_ctr(RESULT_OK_TAG, v, out); }
  int inject_io_err(uint32_t err_tag, Port val, Port& out) {
    Inject in;
    LPort v = ext(val);
    LPort e = err_tag <= IO_ERR_NAME_TAG ? ctr_in(in, err_tag, nullptr, 0) : ctr_in(in, err_tag, &v, 1);
    return commit(in, ctr_in(in, RESULT_ERR_TAG, &e, 1), out);
  }
  int inject_io_err_num(int32_t code, Port& out) { return inject_io_err(IO_ERR_INNER_TAG, new_port(NUM, new_i24(code)), out); }
  int inject_io_err_str(const std::string& msg, Port& out) {
    Port b;
    if (inject_bytes(msg, b)) return -1;
    return inject_io_err(IO_ERR_INNER_TAG, b, out);
  }

  // Readback of a right-nested tuple of at most `size` elements (src/run.c:99-117).
  int read_tup(Port p, uint32_t size, std::vector<Port>& elems) {
    elems.clear();
    while (get_tag(p) == CON && elems.size() + 1 < size) {
      Pair nd = node_load(get_val(p));
      Port e;
      if (expand(get_fst(nd), &e)) return -1;
      elems.push_back(e);
      if (expand(get_snd(nd), &p)) return -1;
    }
    elems.push_back(p);
    return 0;
  }

  // Readback of a lambda-encoded list of u24 (src/run.c:119-182): each
  // element is normalised in turn, the tail booted against ROOT.
  int read_bytes(Port p, std::string& out) {
    out.clear();
    // Most lists are already in normal form: read them on the device in one
    // pass; the host loop below takes over where a REF must be expanded.
    if (normalize()) return -1;
    if (!list_buf) CK(cudaMalloc((void**)&list_buf, (LIST_READ_MAX + 4) * sizeof(uint32_t)));
    read_list_kernel<<<1, 1>>>(d, p, LIST_READ_MAX, list_buf, list_buf + LIST_READ_MAX);
    CK(cudaGetLastError());
    launches++;
    uint32_t info[4];
    CK(cudaMemcpy(info, list_buf + LIST_READ_MAX, sizeof(info), cudaMemcpyDeviceToHost));
    if (info[0]) {
      std::vector<uint32_t> v(info[0]);
      CK(cudaMemcpy(v.data(), list_buf, v.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
      for (uint32_t x : v) out.push_back((char)x);
    }
    d2h_bytes += sizeof(info) + (uint64_t)info[0] * sizeof(uint32_t);
    if (!info[1]) return 0;
    p = (Port)(((uint64_t)info[3] << 32) | info[2]);
    for (;;) {
      if (normalize()) return -1;
      Ctr c;
      if (read_ctr(peek(p), c)) return -1;
      if (c.tag == LIST_CONS_TAG && c.nargs == 2 && get_tag(c.args[0]) == NUM) {
        out.push_back((char)get_u24(get_val(c.args[0])));
        if (boot_root(new_pair(c.args[1], ROOT), ROOT)) return -1;
        p = ROOT;
        continue;
      }
      return 0;
    }
  }

  FILE* io_file(Port p) {
    if (get_tag(p) != NUM) {
      fprintf(stderr, "non-num where file descriptor was expected: %i\n", get_tag(p));
      return nullptr;
    }
    uint32_t fd = get_u24(get_val(p));
    if (fd == 0) return stdin;
    if (fd == 1) return stdout;
    if (fd == 2) return stderr;
    return fd < 256 ? io_files()[fd] : nullptr;
  }
  static FILE** io_files() { static FILE* files[256]; return files; }
  static void** io_dylibs() { static void* libs[256]; return libs; }
  bool io_failed = false;  // set by an hvm_gb300_io_* call that failed inside a DL_CALL
  // The last byte-list readback of the current DL_CALL: a length query and
  // the read that follows evaluate the list once.
  bool io_bytes_valid = false;
  Port io_bytes_port = 0;
  std::string io_bytes;

  // One IO function call (src/run.c:430-770); `ret` receives its result.
  int io_call(const std::string& name, Port argm, Port& ret) {
    std::vector<Port> tup;
    if (name == "READ") {
      if (read_tup(argm, 2, tup)) return -1;
      if (tup.size() != 2) return inject_io_err(IO_ERR_TYPE_TAG, 0, ret);
      FILE* fp = io_file(tup[0]);
      uint32_t want = get_u24(get_val(tup[1]));
      if (!fp) return inject_io_err_num(EBADF, ret);
      std::string buf(want, '\0');
      size_t got = fread(&buf[0], 1, want, fp);
      if (got != want && ferror(fp)) return inject_io_err_num(ferror(fp), ret);
      buf.resize(got);
      Port b;
      if (inject_bytes(buf, b)) return -1;
      return inject_ok(b, ret);
    }
    if (name == "OPEN") {
      if (read_tup(argm, 2, tup)) return -1;
      if (tup.size() != 2) return inject_io_err(IO_ERR_TYPE_TAG, 0, ret);
      std::string path, mode;
      if (read_bytes(tup[0], path) || read_bytes(tup[1], mode)) return -1;
      for (uint32_t fd = 3; fd < 256; fd++) {
        if (io_files()[fd] == nullptr) {
          io_files()[fd] = fopen(path.c_str(), mode.c_str());
          if (!io_files()[fd]) return inject_io_err_num(errno, ret);
          return inject_ok(new_port(NUM, new_u24(fd)), ret);
        }
      }
      return inject_io_err_num(EMFILE, ret);
    }
    if (name == "CLOSE") {
      FILE* fp = io_file(argm);
      if (!fp) return inject_io_err_num(EBADF, ret);
      if (fclose(fp) != 0) return inject_io_err_num(ferror(fp), ret);
      io_files()[get_u24(get_val(argm))] = nullptr;
      return inject_ok(new_port(ERA, 0), ret);
    }
    if (name == "WRITE") {
      if (read_tup(argm, 2, tup)) return -1;
      if (tup.size() != 2) return inject_io_err(IO_ERR_TYPE_TAG, 0, ret);
      FILE* fp = io_file(tup[0]);
      std::string bytes;
      if (read_bytes(tup[1], bytes)) return -1;
      if (!fp) return inject_io_err_num(EBADF, ret);
      if (fwrite(bytes.data(), 1, bytes.size(), fp) != bytes.size()) return inject_io_err_num(ferror(fp), ret);
      return inject_ok(new_port(ERA, 0), ret);
    }
    if (name == "FLUSH") {
      FILE* fp = io_file(argm);
      if (!fp) return inject_io_err_num(EBADF, ret);
      if (fflush(fp) != 0) return inject_io_err_num(ferror(fp), ret);
      return inject_ok(new_port(ERA, 0), ret);
    }
    if (name == "SEEK") {
      if (read_tup(argm, 3, tup)) return -1;
      if (tup.size() != 3) return inject_io_err(IO_ERR_TYPE_TAG, 0, ret);
      FILE* fp = io_file(tup[0]);
      int32_t off = get_i24(get_val(tup[1]));
      uint32_t whence = (uint32_t)get_i24(get_val(tup[2]));
      if (!fp) return inject_io_err_num(EBADF, ret);
      int cw = whence == 0 ? SEEK_SET : whence == 1 ? SEEK_CUR : whence == 2 ? SEEK_END : -1;
      if (cw < 0) return inject_io_err(IO_ERR_TYPE_TAG, 0, ret);
      if (fseek(fp, off, cw) != 0) return inject_io_err_num(ferror(fp), ret);
      return inject_ok(new_port(ERA, 0), ret);
    }
    if (name == "GET_TIME") {
      const uint64_t ns = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
                              std::chrono::system_clock::now().time_since_epoch()).count();
      Inject in;
      LPort t = in.node(ext(new_port(NUM, new_u24((uint32_t)(ns >> 24) & 0xFFFFFFF))),
                        ext(new_port(NUM, new_u24((uint32_t)(ns & 0xFFFFFFF)))));
      Port tp;
      if (commit(in, t, tp)) return -1;
      return inject_ok(tp, ret);
    }
    if (name == "SLEEP") {
      if (read_tup(argm, 2, tup)) return -1;
      if (tup.size() != 2) return inject_io_err(IO_ERR_TYPE_TAG, 0, ret);
      uint64_t ns = ((uint64_t)get_u24(get_val(tup[0])) << 24) | get_u24(get_val(tup[1]));
      struct timespec ts;
      ts.tv_sec = (time_t)(ns / 1000000000ull);
      ts.tv_nsec = (long)(ns % 1000000000ull);
      nanosleep(&ts, nullptr);
      return inject_ok(new_port(ERA, 0), ret);
    }
    if (name == "DL_OPEN") {
      if (read_tup(argm, 2, tup)) return -1;
      std::string path;
      if (read_bytes(tup[0], path)) return -1;
      const int flags = get_u24(get_val(tup.size() > 1 ? tup[1] : 0)) ? RTLD_LAZY : RTLD_NOW;
      for (uint32_t h = 0; h < 256; h++) {
        if (io_dylibs()[h] == nullptr) {
          io_dylibs()[h] = dlopen(path.c_str(), flags);
          if (!io_dylibs()[h]) { const char* e = dlerror(); return inject_io_err_str(e ? e : "dlopen failed", ret); }
          return inject_ok(new_port(NUM, new_u24(h)), ret);
        }
      }
      return inject_io_err_str("too many open dylibs", ret);
    }
    if (name == "DL_CLOSE") {
      if (get_tag(argm) != NUM || get_u24(get_val(argm)) >= 256 || !io_dylibs()[get_u24(get_val(argm))])
        return inject_io_err(IO_ERR_TYPE_TAG, 0, ret);
      void*& h = io_dylibs()[get_u24(get_val(argm))];
      if (dlclose(h) != 0) { const char* e = dlerror(); return inject_io_err_str(e ? e : "dlclose failed", ret); }
      h = nullptr;
      return inject_ok(new_port(ERA, 0), ret);
    }
    if (name == "DL_CALL") {
#ifdef HVM_PORT64
      return inject_io_err_str("DL_CALL needs the 32-bit port build (its library ABI passes 32-bit ports)", ret);
#endif
      // (handle, symbol, argument) (src/run.cu:795-813): the symbol is called
      // as `Port fn(net, arg)` with this runtime as the net handle (the
      // hvm_gb300_io_* functions read and extend the device net); the port it
      // returns is wrapped in Ok.
      if (read_tup(argm, 3, tup)) return -1;
      if (tup.size() != 3) return inject_io_err(IO_ERR_TYPE_TAG, 0, ret);
      if (get_tag(tup[0]) != NUM || get_u24(get_val(tup[0])) >= 256 || !io_dylibs()[get_u24(get_val(tup[0]))])
        return inject_io_err(IO_ERR_TYPE_TAG, 0, ret);
      std::string sym;
      if (read_bytes(tup[1], sym)) return -1;
      dlerror();
      void* f = dlsym(io_dylibs()[get_u24(get_val(tup[0]))], sym.c_str());
      const char* e = dlerror();
      if (e) return inject_io_err_str(e, ret);
      if (!f) return inject_io_err_str("symbol resolves to NULL", ret);
      io_failed = false;
      io_bytes_valid = false;
      const Port r = reinterpret_cast<hvm_gb300_dl_fn>(f)(reinterpret_cast<hvm_gb300_io*>(this), tup[2]);
      if (io_failed) return -1;
      return inject_ok(r, ret);
    }
    return inject_io_err(IO_ERR_NAME_TAG, 0, ret);
  }

  // The IO loop around normalisation (src/run.c:778-810).
  int run_main() {
    if (defs.empty()) return fail("no book loaded");
    if (reset_net()) return -1;
    d.extra_roots = 0;
    if (boot(new_pair(new_port(REF, 0), ROOT))) return -1;
    for (;;) {
      if (normalize()) return -1;
      Ctr c;
      if (read_ctr(peek(ROOT), c)) return -1;
      if (c.nargs < 1 || get_tag(c.args[0]) != CON) break;
      Pair magic = node_load(get_val(c.args[0]));
      if (get_val(get_fst(magic)) != new_u24(IO_MAGIC_0) || get_val(get_snd(magic)) != new_u24(IO_MAGIC_1)) break;
      if (c.tag != IO_CALL_TAG) break;  // IO_DONE
      if (c.nargs != 4) {
        fprintf(stderr, "invalid IO_CALL: args_len = %u\n", c.nargs);
        break;
      }
      const Port argm = c.args[2], cont = c.args[3];
      std::string name;
      if (read_bytes(c.args[1], name)) return -1;
      Port ret;
      if (io_call(name, argm, ret)) return -1;
      Inject in;
      LPort loc = in.node(ext(ret), ext(ROOT));
      Port lp;
      if (commit(in, loc, lp)) return -1;
      if (boot_root(new_pair(lp, cont), ROOT)) return -1;
    }
    return 0;
  }

  // Serialises the tree at ROOT and prints it in the reference's format
  // (src/hvm.c:1535-1699).
  int result_text(std::string& s, Port root = ROOT) {
    if (!g_info) {
      gather_cap = 1u << 24;
      CK(cudaMalloc((void**)&g_out, gather_cap * sizeof(Port)));
      CK(cudaMalloc((void**)&g_kids, gather_cap * sizeof(uint32_t)));
      CK(cudaMalloc((void**)&g_info, 2 * sizeof(uint32_t)));
    }
    gather_kernel<<<1, 1024>>>(d, root, g_out, g_kids, gather_cap, g_info);
    CK(cudaGetLastError());
    launches++;
    uint32_t info[2];
    CK(cudaMemcpy(info, g_info, sizeof(info), cudaMemcpyDeviceToHost));
    d2h_bytes += sizeof(info) + (uint64_t)info[0] * (sizeof(Port) + sizeof(uint32_t));
    if (info[1]) return fail("result tree larger than the readback buffer");
    std::vector<Port> out(info[0]);
    std::vector<uint32_t> kids(info[0]);
    CK(cudaMemcpy(out.data(), g_out, info[0] * sizeof(Port), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(kids.data(), g_kids, info[0] * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    s.clear();
    // Iterative pre-order print; values < 0x100 on the stack are literal chars.
    std::vector<uint64_t> stack;
    stack.push_back(0);
    const uint64_t CHAR = 1ull << 40;
    char buf[64];
    while (!stack.empty()) {
      uint64_t top = stack.back();
      stack.pop_back();
      if (top & CHAR) { s.push_back((char)(top & 0xFF)); continue; }
      uint32_t k = (uint32_t)top;
      Port p = out[k];
      Tag tag = get_tag(p);
      switch (tag) {
        case CON: case DUP: case OPR: case SWI: {
          static const char* open[] = {"(", "{", "$(", "?("};
          static const char close[] = {')', '}', ')', ')'};
          s += open[tag - CON];
          stack.push_back(CHAR | (uint64_t)(unsigned char)close[tag - CON]);
          stack.push_back(kids[k] + 1);
          stack.push_back(CHAR | (uint64_t)' ');
          stack.push_back(kids[k]);
          break;
        }
        case ERA: s += "*"; break;
        case VAR: snprintf(buf, sizeof buf, "x%llx", (unsigned long long)get_val(p)); s += buf; break;
        case NUM: print_numb(get_val(p), s); break;
        case REF: {
          uint32_t fid = get_val(p) & 0xFFFFFFFu;
          s += "@";
          s += fid < defs.size() ? defs[fid].name : std::string("?");
          break;
        }
      }
    }
    return 0;
  }

  static void print_numb(Numb w, std::string& s) {
    static const char* syms[] = {
      "[u24]", "[i24]", "[f24]", "[+]", "[-]", "[:-]", "[*]", "[/]", "[:/]", "[%]", "[:%]",
      "[=]", "[!]", "[<]", "[>]", "[&]", "[|]", "[^]", "[<<]", "[:<<]", "[>>]", "[:>>]"};
    static const char* ops[] = {
      "+", "-", ":-", "*", "/", ":/", "%", ":%", "=", "!", "<", ">", "&", "|", "^", "<<", ":<<", ">>", ":>>"};
    char b[64];
    uint32_t t = get_typ(w);
    if (t == TY_SYM) {
      uint32_t k = get_sym(w);
      s += (k >= 1 && k <= 22) ? syms[k - 1] : "[?]";
    } else if (t == TY_U24) {
      snprintf(b, sizeof b, "%u", get_u24(w)); s += b;
    } else if (t == TY_I24) {
      snprintf(b, sizeof b, "%+d", get_i24(w)); s += b;
    } else if (t == TY_F24) {
      float f = get_f24(w);
      if (isinf(f)) s += signbit(f) ? "-inf" : "+inf";
      else if (isnan(f)) s += "+NaN";
      else { snprintf(b, sizeof b, "%.7e", f); s += b; }
    } else {
      snprintf(b, sizeof b, "[%s0x%07X]", (t >= OP_ADD && t <= FP_SHR) ? ops[t - OP_ADD] : "?", get_u24(w));
      s += b;
    }
  }

  int stats(hvm_gb300_stats* st) {
    Ctl h;
    if (read_ctl(h)) return -1;
    memset(st, 0, sizeof(*st));
    st->itrs = h.itrs;
    st->leak = h.leak;
    st->turns = h.turns;
    st->retries = h.retries;
    for (int i = 0; i < 8; i++) st->rule_hist[i] = h.hist[i];
    for (int i = 0; i < 8; i++) st->prof[i] = h.prof[i];
    st->seconds = norm_seconds;
    st->kernel_ms = kernel_ms;
    st->turn_launches = turn_launches;
    st->launches = launches;
    st->h2d_bytes = h2d_bytes;
    st->d2h_bytes = d2h_bytes;
    st->threads = d.nthreads;
    st->grid = grid;
    st->block = block;
    return 0;
  }
};

HVM_NS_END

// ---- C ABI ---------------------------------------------------------------------------

struct hvm_gb300_runtime {
  hvm::Runtime rt;
};

extern "C" int hvm_gb300_compile_calls(const uint32_t* book, size_t words, char* out, size_t out_cap,
                                       size_t* out_len, char* err, size_t err_cap) {
  auto put_err = [&](const std::string& m) {
    if (err && err_cap) {
      size_t k = std::min(m.size(), err_cap - 1);
      memcpy(err, m.data(), k);
      err[k] = 0;
    }
  };
  hvm::Runtime parser;  // parse_book only: no device state is created
  std::vector<hvm::HostDef> defs;
  if (parser.parse_book(book, words, defs)) { put_err(parser.err); return 1; }
  const std::string src = hvm::compiled_calls_source(defs);
  if (out_len) *out_len = src.size();
  if (out && out_cap > src.size()) { memcpy(out, src.data(), src.size()); out[src.size()] = 0; }
  else if (out) { put_err("output buffer too small"); return 3; }
  return 0;
}

extern "C" void hvm_gb300_default_config(hvm_gb300_config* c) {
  memset(c, 0, sizeof(*c));
  c->device = 0;
  c->threads_per_block = 128;
  c->blocks_per_sm = 0;
  c->node_log2 = 29;
  c->vars_log2 = 29;
  c->ring_log2 = 26;
  c->max_turns = 0;
  c->stop_frac_q8 = 32;
  c->stack_cap = 8;
  c->reg_cap_blocks = 8;
  c->trace_cap = 0;
  c->graph_turns = 0;
  c->node_page_log2 = 0;
  c->var_page_log2 = 0;
  c->max_pages = 0;
  c->steal_min = 0;
  c->turn_budget_cap = 1024;
  c->narrow_below = 1024;
  c->narrow_reg_cap = 0;
  c->rule_select = 1;
  c->fast_calls = 0;
  c->local_nets = 0;
  c->persistent = 0;
  c->upper_half = 0;
}

extern "C" int hvm_gb300_create(const hvm_gb300_config* cfg, hvm_gb300_runtime** out) {
  if (!out) return -1;
  *out = nullptr;
  hvm_gb300_runtime* r = new hvm_gb300_runtime();
  int rc = r->rt.init(cfg);
  *out = r;
  return rc;
}

extern "C" void hvm_gb300_destroy(hvm_gb300_runtime* r) { delete r; }

extern "C" const char* hvm_gb300_error(const hvm_gb300_runtime* r) {
  return r ? r->rt.err.c_str() : "null runtime";
}

extern "C" void hvm_gb300_reset_counters(hvm_gb300_runtime* r) {
  if (r) r->rt.count_reset();
}

extern "C" int hvm_gb300_load_book(hvm_gb300_runtime* r, const uint32_t* book, size_t words) {
  if (!r) return -1;
  r->rt.err.clear();
  return r->rt.load_book(book, words);
}

extern "C" int hvm_gb300_run(hvm_gb300_runtime* r, hvm_gb300_stats* stats) {
  if (!r) return -1;
  r->rt.err.clear();
  if (r->rt.run_main()) return -1;
  if (stats && r->rt.stats(stats)) return -1;
  return 0;
}

extern "C" int hvm_gb300_load_batch(hvm_gb300_runtime* r, const uint32_t* const* books, const size_t* words,
                                    uint32_t n) {
  if (!r) return -1;
  r->rt.err.clear();
  return r->rt.load_batch(books, words, n);
}

extern "C" int hvm_gb300_run_batch(hvm_gb300_runtime* r, hvm_gb300_stats* stats) {
  if (!r) return -1;
  r->rt.err.clear();
  if (r->rt.run_batch()) return -1;
  if (stats && r->rt.stats(stats)) return -1;
  return 0;
}

extern "C" int hvm_gb300_run_stream(hvm_gb300_runtime* r, const double* arrival_s, uint32_t max_inflight,
                                    double live_frac, uint32_t order, double* done_s, uint32_t* result_ports,
                                    hvm_gb300_stats* stats) {
  if (!r || !arrival_s || !done_s || !result_ports) return -1;
  r->rt.err.clear();
  auto t0 = std::chrono::steady_clock::now();
  if (r->rt.run_stream(arrival_s, max_inflight ? max_inflight : 0xFFFFFFFFu, live_frac > 0 ? live_frac : 1.0, done_s,
                       result_ports, order))
    return -1;
  r->rt.norm_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats && r->rt.stats(stats)) return -1;
  return 0;
}

extern "C" int hvm_gb300_set_requests(hvm_gb300_runtime* r, const uint32_t* templates, uint32_t n) {
  if (!r || !templates) return -1;
  r->rt.err.clear();
  return r->rt.set_requests(templates, n);
}

extern "C" int hvm_gb300_batch_roots(hvm_gb300_runtime* r, uint32_t* out, size_t cap) {
  if (!r) return -1;
  if (r->rt.roots.size() != r->rt.nroots) return r->rt.fail("no batch has run");
  if (cap < r->rt.roots.size()) return r->rt.fail("output too small");
  for (size_t i = 0; i < r->rt.roots.size(); i++) {
    const hvm::Port p = r->rt.roots[i];
    if ((uint64_t)p > 0xFFFFFFFFull) return r->rt.fail("a root port does not fit 32 bits (use hvm_gb300_batch_result)");
    out[i] = (uint32_t)p;
  }
  return 0;
}

extern "C" int hvm_gb300_batch_result(hvm_gb300_runtime* r, uint32_t net, char* out, size_t cap, size_t* len) {
  if (!r) return -1;
  if (net >= r->rt.nroots) return r->rt.fail("net index out of range");
  std::string s;
  if (r->rt.result_text(s, hvm::new_port(hvm::VAR, hvm::ROOT_VAR - net))) return -1;
  if (len) *len = s.size();
  if (out) {
    if (cap <= s.size()) { r->rt.fail("result buffer too small"); return -2; }
    memcpy(out, s.data(), s.size());
    out[s.size()] = 0;
  }
  return 0;
}

extern "C" int hvm_gb300_count_live(hvm_gb300_runtime* r, uint64_t* out3) {  // out3: 5 words
  if (!r || !out3) return -1;
  hvm::Runtime& rt = r->rt;
  unsigned long long* dev = nullptr;
  if (cudaMalloc(&dev, 3 * sizeof(unsigned long long)) != cudaSuccess) return rt.fail("cudaMalloc failed");
  cudaMemset(dev, 0, 3 * sizeof(unsigned long long));
  hvm::count_live_kernel<<<1024, 256>>>(rt.d, 1ull << rt.cfg.node_log2, 1ull << rt.cfg.vars_log2, dev);
  unsigned long long h[3] = {0, 0, 0};
  cudaError_t e = cudaMemcpy(h, dev, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(dev);
  if (e != cudaSuccess) return rt.fail(cudaGetErrorString(e));
  hvm::Ctl c;
  if (rt.read_ctl(c)) return -1;
  out3[0] = h[0]; out3[1] = h[1]; out3[2] = h[2];
  out3[3] = c.npool_next; out3[4] = c.vpool_next;
  return 0;
}

extern "C" int hvm_gb300_trace(hvm_gb300_runtime* r, hvm_gb300_turn* out, size_t cap, size_t* n) {
  if (!r) return -1;
  hvm::Ctl h;
  if (r->rt.read_ctl(h)) return -1;
  size_t have = h.turns < r->rt.cfg.trace_cap ? (size_t)h.turns : (size_t)r->rt.cfg.trace_cap;
  if (n) *n = have;
  if (!out || !r->rt.mem_trace) return 0;
  size_t k = have < cap ? have : cap;
  std::vector<hvm::TurnRecord> tmp(k);
  if (k && cudaMemcpy(tmp.data(), r->rt.mem_trace, k * sizeof(hvm::TurnRecord), cudaMemcpyDeviceToHost) != cudaSuccess)
    return r->rt.fail("trace copy failed");
  for (size_t i = 0; i < k; i++) {
    out[i].t_ns = tmp[i].t_ns;
    out[i].live_nodes = tmp[i].live_nodes;
    out[i].itrs = tmp[i].itrs;
    out[i].pending = tmp[i].pending;
    out[i].dry = tmp[i].dry;
    out[i].stopped = tmp[i].stopped;
    out[i].budget = tmp[i].budget;
    out[i].per_thread = tmp[i].per_thread;
    for (int j = 0; j < 16; j++) out[i].features[j] = tmp[i].features[j];
    for (int j = 0; j < 3; j++) out[i].outputs[j] = tmp[i].outputs[j];
  }
  return 0;
}

extern "C" int hvm_gb300_set_policy(hvm_gb300_runtime* r, uint32_t mode, const float* weights, size_t n_weights,
                                    const float* constants) {
  if (!r) return -1;
  r->rt.err.clear();
  return r->rt.set_policy(mode, weights, n_weights, constants);
}

extern "C" int hvm_gb300_result(hvm_gb300_runtime* r, char* out, size_t cap, size_t* len) {
  if (!r) return -1;
  hvm::Runtime& rt = r->rt;
  if (!rt.result_valid) {  // computed once per run: a size query and the copy share it
    if (rt.result_text(rt.result_cache)) return -1;
    rt.result_valid = true;
  }
  const std::string& s = rt.result_cache;
  if (len) *len = s.size();
  if (out) {
    if (cap <= s.size()) { r->rt.fail("result buffer too small"); return -2; }
    memcpy(out, s.data(), s.size());
    out[s.size()] = 0;
  }
  return 0;
}

// ---- Net access for DL_CALL libraries ------------------------------------------------
// The host-side net functions the reference's run-cu exports to the libraries
// a DL_CALL names (src/hvm.cu:1842-1893, src/run.cu:102-285), over the device
// net of the runtime running the IO loop. A failure records the error, makes
// the DL_CALL fail and returns -1.

static hvm::Runtime& io_rt(hvm_gb300_io* io) { return *reinterpret_cast<hvm::Runtime*>(io); }
// The ports these functions exchange are 32-bit: the 64-bit port build calls
// no DL_CALL library, so there they refuse.
constexpr bool IO_PORTS_32 = hvm::PORT_BITS == 32;
static int io_fail(hvm::Runtime& rt, const char* msg) {
  if (msg) rt.fail(msg);
  rt.io_failed = true;
  return -1;
}

extern "C" int hvm_gb300_io_expand(hvm_gb300_io* io, uint32_t port, uint32_t* out) {
  if (!IO_PORTS_32) return -1;
  using namespace hvm;
  if (!io || !out) return -1;
  hvm::Runtime& rt = io_rt(io);
  rt.io_bytes_valid = false;  // the net changes
  Port p;
  if (rt.expand(port, &p)) return io_fail(rt, nullptr);
  *out = p;
  return 0;
}

extern "C" int hvm_gb300_io_node_load(hvm_gb300_io* io, uint32_t port, uint32_t* fst, uint32_t* snd) {
  if (!IO_PORTS_32) return -1;
  using namespace hvm;
  if (!io || !fst || !snd) return -1;
  hvm::Runtime& rt = io_rt(io);
  const uint32_t tag = get_tag(port);
  if (tag < CON || get_val(port) > rt.d.node_mask) return io_fail(rt, "hvm_gb300_io_node_load: not a node port");
  const Pair n = rt.node_load(get_val(port));
  *fst = get_fst(n);
  *snd = get_snd(n);
  return 0;
}

extern "C" int hvm_gb300_io_make_node(hvm_gb300_io* io, uint32_t tag, uint32_t fst, uint32_t snd, uint32_t* out) {
  if (!IO_PORTS_32) return -1;
  using namespace hvm;
  if (!io || !out) return -1;
  hvm::Runtime& rt = io_rt(io);
  rt.io_bytes_valid = false;  // the net changes
  if (tag < CON || tag > SWI) return io_fail(rt, "hvm_gb300_io_make_node: not a node tag");
  hvm::Runtime::Inject in;
  const hvm::Runtime::LPort n = in.node(hvm::Runtime::ext(fst), hvm::Runtime::ext(snd));
  Port p;
  if (rt.commit(in, n, p)) return io_fail(rt, nullptr);
  *out = new_port(tag, get_val(p));
  return 0;
}

extern "C" int hvm_gb300_io_readback_tup(hvm_gb300_io* io, uint32_t port, uint32_t size, uint32_t* elems,
                                         uint32_t* n) {
  if (!IO_PORTS_32) return -1;
  using namespace hvm;
  if (!io || !elems || !n || size == 0) return -1;
  hvm::Runtime& rt = io_rt(io);
  rt.io_bytes_valid = false;  // the net changes
  std::vector<Port> tup;
  if (rt.read_tup(port, size, tup)) return io_fail(rt, nullptr);
  for (size_t i = 0; i < tup.size(); i++) elems[i] = tup[i];
  *n = (uint32_t)tup.size();
  return 0;
}

extern "C" int hvm_gb300_io_readback_bytes(hvm_gb300_io* io, uint32_t port, uint8_t* out, size_t cap, size_t* len) {
  if (!IO_PORTS_32) return -1;
  using namespace hvm;
  if (!io || !len) return -1;
  hvm::Runtime& rt = io_rt(io);
  if (!rt.io_bytes_valid || rt.io_bytes_port != port) {
    rt.io_bytes_valid = false;
    if (rt.read_bytes(port, rt.io_bytes)) return io_fail(rt, nullptr);
    rt.io_bytes_valid = true;
    rt.io_bytes_port = port;
  }
  const std::string& b = rt.io_bytes;
  *len = b.size();
  if (out) {
    if (cap < b.size()) return io_fail(rt, "hvm_gb300_io_readback_bytes: buffer too small");
    memcpy(out, b.data(), b.size());
  }
  return 0;
}

extern "C" int hvm_gb300_io_inject_bytes(hvm_gb300_io* io, const uint8_t* bytes, size_t len, uint32_t* out) {
  if (!IO_PORTS_32) return -1;
  using namespace hvm;
  if (!io || !out || (len && !bytes)) return -1;
  hvm::Runtime& rt = io_rt(io);
  rt.io_bytes_valid = false;  // the net changes
  Port p;
  if (rt.inject_bytes(std::string((const char*)bytes, len), p)) return io_fail(rt, nullptr);
  *out = p;
  return 0;
}

extern "C" int hvm_gb300_wait_probe(int32_t device, uint32_t limit_ms, uint32_t* timed_out, double* waited_ms) {
  if (!timed_out || !waited_ms || limit_ms == 0 || limit_ms > 10000) return -1;
  if (cudaSetDevice(device) != cudaSuccess) return -1;
  unsigned* buf = nullptr;
  if (cudaMalloc((void**)&buf, 4 * sizeof(unsigned)) != cudaSuccess) return -1;
  int rc = cudaMemset(buf, 0, 4 * sizeof(unsigned)) == cudaSuccess ? 0 : -1;
  if (rc == 0) {
    hvm::wait_probe_kernel<<<1, 1>>>(buf, (unsigned long long)limit_ms * 1000000ull, buf + 1);
    unsigned out[3] = {0, 0, 0};
    rc = cudaGetLastError() == cudaSuccess && cudaMemcpy(out, buf + 1, sizeof(out), cudaMemcpyDeviceToHost) == cudaSuccess
             ? 0 : -1;
    *timed_out = out[0];
    *waited_ms = (double)(((unsigned long long)out[2] << 32) | out[1]) / 1e6;
  }
  cudaFree(buf);
  return rc;
}

// Drop-in for the reference's CUDA entry point (src/hvm.cu:2320-2397): loads
// the book, normalises @main and prints `Result:`, `- ITRS`, `- LEAK`,
// `- TIME` and `- MIPS` on stdout.
extern "C" void hvm_cu(const uint32_t* book_buffer) {
  hvm_gb300_runtime* r = nullptr;
  if (hvm_gb300_create(nullptr, &r) != 0) {
    fprintf(stderr, "Failed to initialise the GB300 runtime: %s\n", r ? hvm_gb300_error(r) : "?");
    hvm_gb300_destroy(r);
    exit(EXIT_FAILURE);
  }
  if (hvm_gb300_load_book(r, book_buffer, 0) != 0) {
    fprintf(stderr, "%s\n", hvm_gb300_error(r));
    fprintf(stderr, "failed to load book\n");
    hvm_gb300_destroy(r);
    return;
  }
  auto t0 = std::chrono::steady_clock::now();
  hvm_gb300_stats st;
  if (hvm_gb300_run(r, &st) != 0) {
    fprintf(stderr, "Failed to run the net: %s\n", hvm_gb300_error(r));
    hvm_gb300_destroy(r);
    exit(EXIT_FAILURE);
  }
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::string s;
  if (r->rt.result_text(s) != 0) {
    fprintf(stderr, "Failed to read back the result: %s\n", hvm_gb300_error(r));
    hvm_gb300_destroy(r);
    exit(EXIT_FAILURE);
  }
  printf("Result: %s\n", s.c_str());
  printf("- ITRS: %llu\n", (unsigned long long)st.itrs);
  printf("- LEAK: %llu\n", (unsigned long long)st.leak);
  printf("- TIME: %.2fs\n", secs);
  printf("- MIPS: %.2f\n", (double)st.itrs / secs / 1000000.0);
  fflush(stdout);
  hvm_gb300_destroy(r);
}

// ---- Allocation-free evaluation ------------------------------------------------------
//
// hvm_gb300_run_noalloc evaluates a small net without allocating any memory:
// the whole net (node and var spaces, redex ring, page lists, control block,
// book tables and the readback buffers) lives in one fixed device array of
// NOALLOC_ARENA_BYTES. It serves callers that may not call cudaMalloc — a
// host whose device memory is owned by another allocator or a pool that must
// not fragment, or an embedding that has to guarantee the call cannot fail on
// allocation. Its copies, memsets and launches are synchronous calls on the
// default stream. The array is held by every GPU that loads the library until the
// process exits. All calls share it, so calls that overlap on the GPU race
// with each other; each call clears what must start at zero before it runs.
// The first call on a device resolves the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture.

HVM_NS_BEGIN
namespace noalloc {

// Fixed capacities of the arena. The grid is fixed (16 blocks of 128 threads,
// enough for small nets) so the page layout is fixed: 256-word pages, up to
// 32 pages of each kind per thread.
constexpr uint32_t BLOCKS = 16, THREADS = 128, NTHREADS = BLOCKS * THREADS, CAP = 8;
constexpr uint32_t NODE_LOG2 = 20, VARS_LOG2 = 20, RING_LOG2 = 18, PAGE_LOG2 = 8, LIST_PAGES = 32;
constexpr uint32_t MAX_BOOK_WORDS = 1u << 19, MAX_DEFS = 4096, MAX_PAIRS = 1u << 18;
constexpr uint32_t MAX_DEF_NODES = 32, MAX_DEF_VARS = 32, MAX_TREE = 1u << 16;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t OFF_NODE = 0;
constexpr size_t OFF_VARS = OFF_NODE + align256(sizeof(Pair) << NODE_LOG2);
constexpr size_t OFF_RING = OFF_VARS + align256(sizeof(Port) << VARS_LOG2);
constexpr size_t OFF_LISTS = OFF_RING + align256(sizeof(Pair) << RING_LOG2);
constexpr size_t LISTS_WORDS = 2ull * NTHREADS * (LIST_PAGES + 3);
constexpr size_t OFF_RAW = OFF_LISTS + align256(LISTS_WORDS * sizeof(uint32_t));
constexpr size_t OFF_DEFS = OFF_RAW + align256((size_t)MAX_BOOK_WORDS * sizeof(uint32_t));
constexpr size_t OFF_RAWPOS = OFF_DEFS + align256((size_t)MAX_DEFS * sizeof(DefHdr));
constexpr size_t OFF_BOOK = OFF_RAWPOS + align256((size_t)MAX_DEFS * sizeof(uint32_t));
constexpr size_t OFF_OUT = OFF_BOOK + align256((size_t)MAX_PAIRS * sizeof(Pair));
constexpr size_t OFF_KIDS = OFF_OUT + align256((size_t)MAX_TREE * sizeof(Port));
constexpr size_t OFF_INFO = OFF_KIDS + align256((size_t)MAX_TREE * sizeof(uint32_t));
constexpr size_t OFF_CTL = OFF_INFO + 256;
constexpr size_t ARENA_BYTES = OFF_CTL + align256(sizeof(Ctl));

}  // namespace noalloc
HVM_NS_END

// The arena. In host code this name is a host-side stand-in, not a device
// address: only the address from cudaGetSymbolAddress may be given to kernels.
static __device__ __align__(256) unsigned char g_noalloc_arena[hvm::noalloc::ARENA_BYTES];

HVM_NS_BEGIN
namespace noalloc {

constexpr int MAX_DEVICES = 64;
static unsigned char* g_arena_dev[MAX_DEVICES];  // device address of the arena, per device
static std::mutex g_arena_mu;                    // guards g_arena_dev (first calls from several threads)

// Builds the device book tables from the raw buffer already in the arena:
// thread 0 lays out the def headers (the host has validated the buffer),
// then all threads copy each def's pairs to an 8-byte aligned table.
__global__ void book_kernel(const uint32_t* raw, DefHdr* defs, uint32_t* rawpos, Pair* book) {
  if (threadIdx.x == 0) {
    uint32_t ndefs = raw[0], at = 1, off = 0;
    for (uint32_t k = 0; k < ndefs; k++) {
      uint32_t fid = raw[at];
      uint32_t safe = raw[at + 65], rl = raw[at + 66], nl = raw[at + 67], vl = raw[at + 68];
      defs[fid] = DefHdr{nl, rl, vl, safe ? 1u : 0u, raw[at + 69], off, 0, 0};
      rawpos[fid] = at + DEF_HEADER_WORDS;
      off += rl + nl;
      at += DEF_HEADER_WORDS + 2 * (rl + nl);
    }
  }
  __syncthreads();
  uint32_t ndefs = raw[0];
  for (uint32_t f = 0; f < ndefs; f++) {
    const DefHdr h = defs[f];
    const uint32_t* src = raw + rawpos[f];
    for (uint32_t i = threadIdx.x; i < h.rbag_len + h.node_len; i += blockDim.x) {
      book[h.off + i] = new_pair(src[2 * i], src[2 * i + 1]);
    }
  }
}

struct Ctx {
  Dev d;
  unsigned char* arena;
  char* err;
  size_t err_cap;
};

static int failf(Ctx& x, const char* msg, long long a = -1) {
  if (x.err && x.err_cap) {
    if (a >= 0) snprintf(x.err, x.err_cap, "%s (%lld)", msg, a);
    else snprintf(x.err, x.err_cap, "%s", msg);
  }
  return -1;
}

static int cuda_ok(Ctx& x, cudaError_t e) {
  if (e == cudaSuccess) return 0;
  return failf(x, cudaGetErrorString(e));
}

static int read_ctl(Ctx& x, Ctl& h) { return cuda_ok(x, cudaMemcpy(&h, x.d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost)); }

static int normalize(Ctx& x) {
  Ctl h;
  uint32_t batch = 4;
  unsigned long long last_itrs = ~0ull, last_pending = ~0ull;
  uint64_t stalled = 0, turns = 0;
  for (;;) {
    for (uint32_t i = 0; i < batch; i++) turn_kernel<8, false, false, false><<<BLOCKS, THREADS, (size_t)THREADS * CAP * sizeof(Pair)>>>(x.d, CAP);
    if (cuda_ok(x, cudaGetLastError()) || read_ctl(x, h)) return -1;
    turns += batch;
    if (h.status) return failf(x, status_text(h.status), h.err_info);
    if (h.base == h.in_end) return 0;
    if (h.itrs == last_itrs && h.pending == last_pending) {
      if (++stalled > 4096) return failf(x, "no progress: interaction count stalled with redexes pending");
    } else {
      stalled = 0;
    }
    if (turns > (1ull << 24)) return failf(x, "turn budget exhausted before normal form");
    last_itrs = h.itrs;
    last_pending = h.pending;
    if (batch < 64) batch *= 2;
  }
}

static int boot(Ctx& x, Pair redex) {
  boot_kernel<<<1, 1>>>(x.d, redex, get_snd(redex), CAP);
  return cuda_ok(x, cudaGetLastError());
}

static int vars_load(Ctx& x, uint32_t i, Port& v) {
  return cuda_ok(x, cudaMemcpy(&v, x.d.vars + (i & x.d.vars_mask), sizeof(Port), cudaMemcpyDeviceToHost));
}
static int vars_store(Ctx& x, uint32_t i, Port v) {
  return cuda_ok(x, cudaMemcpy(x.d.vars + (i & x.d.vars_mask), &v, sizeof(Port), cudaMemcpyHostToDevice));
}
static int node_load(Ctx& x, uint32_t i, Pair& v) {
  return cuda_ok(x, cudaMemcpy(&v, x.d.node + i, sizeof(Pair), cudaMemcpyDeviceToHost));
}

// Read-only chase (src/hvm.c:781-790).
static int peek(Ctx& x, Port p, Port& out) {
  while (get_tag(p) == VAR) {
    Port v;
    if (vars_load(x, get_val(p), v)) return -1;
    if (v == NONE || v == 0) break;
    p = v;
  }
  out = p;
  return 0;
}

// Normalises every REF the readback meets (src/hvm.c:1233-1243).
static int expand(Ctx& x, Port p, Port& out) {
  Port saved, got;
  if (vars_load(x, ROOT_VAR, saved) || peek(x, p, got)) return -1;
  while (get_tag(got) == REF) {
    Port r;
    if (boot(x, new_pair(got, ROOT)) || normalize(x) || vars_load(x, ROOT_VAR, r) || peek(x, r, got)) return -1;
  }
  if (vars_store(x, ROOT_VAR, saved)) return -1;
  out = got;
  return 0;
}

// The IO loop's constructor walk (src/run.c:65-97, 778-810). A normal form
// that asks for an IO call is refused: this entry point has no IO layer.
static int readback_walk(Ctx& x) {
  Port root, lam, app, arg, first = 0;
  Pair n;
  uint32_t tag, nargs = 0;
  if (peek(x, ROOT, root) || expand(x, root, lam)) return -1;
  if (get_tag(lam) != CON) return 0;
  if (node_load(x, get_val(lam), n) || expand(x, get_fst(n), app)) return -1;
  if (get_tag(app) != CON) return 0;
  Pair app_n;
  if (node_load(x, get_val(app), app_n) || expand(x, get_fst(app_n), arg)) return -1;
  if (get_tag(arg) != NUM) return 0;
  tag = get_u24(get_val(arg));
  for (;;) {
    if (expand(x, get_snd(app_n), app)) return -1;
    if (get_tag(app) != CON) break;
    if (node_load(x, get_val(app), app_n) || expand(x, get_fst(app_n), arg)) return -1;
    if (nargs++ == 0) first = arg;
  }
  if (tag == IO_CALL_TAG && nargs >= 1 && get_tag(first) == CON) {
    Pair magic;
    if (node_load(x, get_val(first), magic)) return -1;
    if (get_val(get_fst(magic)) == new_u24(IO_MAGIC_0) && get_val(get_snd(magic)) == new_u24(IO_MAGIC_1))
      return failf(x, "IO calls are not supported by hvm_gb300_run_noalloc");
  }
  return 0;
}

// Checks the caller's book in place against the arena's limits and the
// reference loader's limits (src/hvm.c:1408-1453); ports must stay inside
// their definition.
static int validate(Ctx& x, const uint32_t* w, size_t words) {
  if (!w || words < 1) return failf(x, "empty book buffer");
  if (words > MAX_BOOK_WORDS) return failf(x, "book larger than the fixed arena allows (words)", (long long)words);
  uint32_t ndefs = w[0];
  if (ndefs == 0 || ndefs > MAX_DEFS) return failf(x, "book has more definitions than the fixed arena allows", ndefs);
  size_t at = 1, pairs = 0;
  uint32_t seen[MAX_DEFS / 32] = {0};  // every fid exactly once
  for (uint32_t k = 0; k < ndefs; k++) {
    if (at + DEF_HEADER_WORDS > words) return failf(x, "failed to load book: truncated");
    uint32_t fid = w[at], rl = w[at + 66], nl = w[at + 67], vl = w[at + 68];
    if (fid >= ndefs) return failf(x, "failed to load book: bad definition id", fid);
    if (seen[fid / 32] & (1u << (fid % 32))) return failf(x, "failed to load book: duplicate definition id", fid);
    seen[fid / 32] |= 1u << (fid % 32);
    if (rl > DEF_RBAG_LEN) return failf(x, "definition has too many redexes", rl);
    if (nl > MAX_DEF_NODES) return failf(x, "definition has more nodes than the fixed arena allows", nl);
    if (vl > MAX_DEF_VARS) return failf(x, "definition has more vars than the fixed arena allows", vl);
    size_t end = at + DEF_HEADER_WORDS + 2ull * (rl + nl);
    if (end > words) return failf(x, "failed to load book: truncated");
    auto ok = [&](Port p) {
      Tag t = get_tag(p);
      if (t >= CON) return get_val(p) < nl;
      if (t == VAR) return get_val(p) < vl;
      if (t == REF) return (get_val(p) & 0xFFFFFFFu) < ndefs;
      return true;
    };
    bool good = ok(w[at + 69]);
    for (size_t i = at + DEF_HEADER_WORDS; i < end; i++) good = good && ok(w[i]);
    if (!good) return failf(x, "failed to load book: a port points outside its definition", fid);
    pairs += rl + nl;
    at = end;
  }
  if (pairs > MAX_PAIRS) return failf(x, "book has more pairs than the fixed arena allows", (long long)pairs);
  return 0;
}

}  // namespace noalloc
HVM_NS_END

extern "C" int hvm_gb300_run_noalloc(const uint32_t* book, size_t words, uint32_t* out_ports, uint32_t* out_kids,
                                     size_t out_cap, size_t* out_len, uint64_t* out_itrs, char* err, size_t err_cap) {
  using namespace hvm;
  using namespace hvm::noalloc;
  Ctx x{};
  x.err = err;
  x.err_cap = err_cap;
  if (PORT_BITS != 32) return failf(x, "hvm_gb300_run_noalloc returns 32-bit ports: not in the 64-bit port build");
  if (err && err_cap) err[0] = 0;
  int dev = 0;
  if (cuda_ok(x, cudaGetDevice(&dev))) return -1;
  if (dev < 0 || dev >= MAX_DEVICES) return failf(x, "device ordinal out of range", dev);
  unsigned char* A = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_arena_mu);
    if (!g_arena_dev[dev]) {
      void* p = nullptr;
      if (cuda_ok(x, cudaGetSymbolAddress(&p, g_noalloc_arena))) return -1;
      g_arena_dev[dev] = (unsigned char*)p;
    }
    A = g_arena_dev[dev];
  }
  x.arena = A;
  if (validate(x, book, words)) return -1;

  // Device view of the arena.
  Dev& d = x.d;
  d.node = (Pair*)(A + OFF_NODE);
  d.vars = (Port*)(A + OFF_VARS);
  d.vars_mask = (1u << VARS_LOG2) - 1;
  d.node_mask = (1u << NODE_LOG2) - 1;
  d.ring = (Pair*)(A + OFF_RING);
  d.ring_mask = (1ull << RING_LOG2) - 1;
  uint32_t* lw = (uint32_t*)(A + OFF_LISTS);
  for (PagedSpace* sp : {&d.nspace, &d.vspace}) {
    sp->page_log2 = PAGE_LOG2;
    sp->max_pages = LIST_PAGES;
    sp->lists = lw; lw += (size_t)NTHREADS * LIST_PAGES;
    sp->counts = lw; lw += NTHREADS;
    sp->pos = lw; lw += NTHREADS;
    sp->off = lw; lw += NTHREADS;
  }
  d.npool_base = reserved_pages(PAGE_LOG2);
  d.vpool_base = reserved_pages(PAGE_LOG2);
  d.npool_end = 1u << (NODE_LOG2 - PAGE_LOG2);
  d.vpool_end = 1u << (VARS_LOG2 - PAGE_LOG2);
  d.nloc = nullptr;  // every def fits one chunk: the scratch tables are never used
  d.vloc = nullptr;
  d.nthreads = NTHREADS;
  d.steal_min = 2;
  d.ndefs = book[0];
  d.defs = (const DefHdr*)(A + OFF_DEFS);
  d.book = (const Pair*)(A + OFF_BOOK);
  d.ctl = (Ctl*)(A + OFF_CTL);

  // Book: raw words in, then the device tables.
  if (cuda_ok(x, cudaMemcpy(A + OFF_RAW, book, words * sizeof(uint32_t), cudaMemcpyHostToDevice))) return -1;
  book_kernel<<<1, 256>>>((const uint32_t*)(A + OFF_RAW), (DefHdr*)(A + OFF_DEFS), (uint32_t*)(A + OFF_RAWPOS),
                          (Pair*)(A + OFF_BOOK));
  if (cuda_ok(x, cudaGetLastError())) return -1;

  // Clear what must start at zero: the net, the control block.
  if (cuda_ok(x, cudaMemset(A + OFF_NODE, 0, sizeof(Pair) << NODE_LOG2)) ||
      cuda_ok(x, cudaMemset(A + OFF_VARS, 0, sizeof(Port) << VARS_LOG2)) ||
      cuda_ok(x, cudaMemset(A + OFF_CTL, 0, sizeof(Ctl)))) return -1;
  uint32_t frac = 128;
  if (cuda_ok(x, cudaMemcpy(&d.ctl->stop_frac_q8, &frac, sizeof(frac), cudaMemcpyHostToDevice))) return -1;
  reset_alloc_kernel<<<(NTHREADS + 255) / 256, 256>>>(d);
  if (cuda_ok(x, cudaGetLastError())) return -1;

  // Boot @main ~ ROOT, normalise, run the readback expansion.
  if (boot(x, new_pair(new_port(REF, 0), ROOT)) || normalize(x) || readback_walk(x)) return -1;

  // Serialise the normal form into the caller's arrays.
  uint32_t* info = (uint32_t*)(A + OFF_INFO);
  gather_kernel<<<1, 1024>>>(d, ROOT, (Port*)(A + OFF_OUT), (uint32_t*)(A + OFF_KIDS), MAX_TREE, info);
  if (cuda_ok(x, cudaGetLastError())) return -1;
  uint32_t hinfo[2];
  if (cuda_ok(x, cudaMemcpy(hinfo, info, sizeof(hinfo), cudaMemcpyDeviceToHost))) return -1;
  if (hinfo[1]) return failf(x, "normal form larger than the fixed arena's readback buffer", MAX_TREE);
  if (out_len) *out_len = hinfo[0];
  if (hinfo[0] > out_cap) return failf(x, "output arrays too small for the normal form", hinfo[0]);
  if (out_ports && cuda_ok(x, cudaMemcpy(out_ports, A + OFF_OUT, hinfo[0] * sizeof(Port), cudaMemcpyDeviceToHost)))
    return -1;
  if (out_kids && cuda_ok(x, cudaMemcpy(out_kids, A + OFF_KIDS, hinfo[0] * sizeof(uint32_t), cudaMemcpyDeviceToHost)))
    return -1;
  Ctl h;
  if (read_ctl(x, h)) return -1;
  if (out_itrs) *out_itrs = h.itrs;
  return 0;
}
