// evaluator.cuh — device side of the GB300 HVM2 evaluator: net memory
// access, allocation, the lock-free linker and the eight interaction rules.
//
// The rules, the linker and the interaction count follow the reference
// semantics exactly (src/hvm.c:784-1122; src/hvm.cu:999-1420), because the
// normal form and the total interaction count must equal `hvm run-c`'s. What
// differs is the GB300 execution model around them:
//   * every net word lives in HBM and is touched only at L2 (ld.cg/st.cg and
//     atomics), so no SM ever reads a stale L1 copy of a shared word;
//   * a thread publishes freshly created nodes/vars with one gpu-scope fence
//     before its first link, instead of the reference's per-access
//     availability re-tries (the re-try path is kept as a safety net);
//   * redexes live in a per-thread LIFO in shared memory; overflow and the
//     end-of-turn remainder go to one global ring (see runtime.cu);
//   * allocation scans a per-thread slice of the node/var space for free
//     (zero) words, as the reference does (src/hvm.cu:880-912), with a bound
//     on the scan that turns exhaustion into an error status instead of a
//     spin.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "hvm_defs.h"

HVM_NS_BEGIN

// Device status codes (0 = running / ok). Written once, first error wins.
enum : uint32_t {
  ST_OK = 0,
  ST_OOM_NODES = 1,     // no free node/var word: page list full or page pool empty
  ST_OOM_VARS = 2,      // (reserved)
  ST_RING_FULL = 3,     // the global redex ring overflowed
  ST_LINK_UNSET = 4,    // a link met a var word that was never created
  ST_LINK_LIMIT = 5,    // a substitution chain exceeded the iteration bound
  ST_BAD_REF = 6,       // a REF to a definition the book does not have
  ST_DRAIN = 7,         // a turn's end could not make its local net global within the bound
  ST_WAIT = 8,          // persistent launch: a block waited too long for a turn to close
};

// One book definition on the device. Pairs for a def are stored at
// book[off .. off+rbag_len) (redexes) then book[off+rbag_len ..) (nodes).
struct DefHdr {
  uint32_t node_len, rbag_len, vars_len, safe;
  uint32_t root, off;
  uint32_t joined;  // 1: the rbag holds every link of a call, the root's included
                    // (its caller end written as CALLER_PORT), with vars that
                    // only wired two links removed; 0: the book's own layout
  uint32_t fast;    // CALL-time fast paths (src/cmp.rs:110-290), see fast_kind()
};

// DefHdr::fast, for joined defs whose root is a CON node (the root link is
// then the last link) of at most 32 nodes and vars. Bits 0-1: 0 none,
// FAST_ANNI (the root CON meets a CON caller), FAST_SWITCH (the root is
// `(?((s1 s2) r) r)`: a switch whose result is the call's result, fed by a
// caller `(#X R)`); bits 2-6 the root node, 7-11 the switch node, 12-16 its
// CON node, 17-21 the var r. The def's table then holds two more pairs after
// its nodes: the root's two ports, and (s1, s2).
constexpr uint32_t FAST_ANNI = 1, FAST_SWITCH = 2;
__host__ __device__ __forceinline__ uint32_t fast_kind(uint32_t f) { return f & 3u; }
__host__ __device__ __forceinline__ uint32_t fast_field(uint32_t f, int k) { return (f >> (2 + 5 * k)) & 31u; }

// Stands for the other side of a CALL's redex in a joined def's link list
// (a REF to a fid no book can have).
constexpr Port CALLER_PORT = 0xFFFFFFF9u;

// One record per completed turn, written by the turn's last block.
struct TurnRecord {
  unsigned long long t_ns;          // %globaltimer when the turn closed
  long long live_nodes;             // node words in use after the turn
  unsigned long long itrs;          // cumulative interactions
  unsigned long long pending;       // redexes in the ring for the next turn
  unsigned int dry, stopped;        // dry threads at close; 1 if ended by the dry rule
  unsigned int budget, per_thread;  // the closed turn's budget and static share
  float features[16];               // scheduler inputs computed at the close of the turn
  float outputs[3];                 // the next turn's parameters in output space (see apply_policy)
};

// Control block of one net. Hot atomics sit on separate 128-byte lines.
struct alignas(128) Ctl {
  unsigned long long head;          // next dynamically claimable ring index
  unsigned long long pad_h[15];
  unsigned long long tail;          // next free ring index
  unsigned long long pad_t[15];
  unsigned long long base;          // first ring index of this turn's input
  unsigned long long in_end;        // one past the last input index
  unsigned long long itrs;          // counted interactions (all turns)
  unsigned long long leak;          // redexes that went through the ring
  unsigned long long retries;       // availability re-tries (diagnostic)
  unsigned long long turns;         // completed turns
  unsigned long long pending;       // redexes left after the last turn
  unsigned long long pad_p[7];
  unsigned int dry;                 // threads that ran out of work this turn
  unsigned int stop;                // set once enough threads are dry: end the turn
  unsigned int stop_at;             // dry count that sets `stop`
  unsigned int stop_frac_q8;        // end a turn once busy < (1 - frac) * initially busy
  unsigned int pad_s[28];
  unsigned int blocks_done;
  unsigned int status;
  unsigned int err_info;
  unsigned int static_per_thread;   // ring items each thread takes at turn start
  unsigned int budget;              // interactions per thread per turn
  unsigned int chunk;               // items per dynamic claim
  unsigned int budget_cap;          // 0, or the most rounds a turn may run (bounds how long the
                                    // host waits between admissions and completion checks)
  unsigned int pad_c[1];
  unsigned long long hist[8];       // interactions per rule (diagnostic)
  unsigned long long prof[8];       // profile counters (when prof_on): see PROF_*
  unsigned int prof_on;
  unsigned int oom_space, oom_pages, oom_dry, oom_pool_dry;  // diagnostics of the first out-of-memory
  // Free-page rings (node, var): pages returned by lanes that found them
  // empty. Taken from [head, end) during a turn, returned at tail; `end`
  // moves to `tail` between turns (the redex ring's discipline).
  unsigned int nf_head, nf_tail, nf_end, vf_head, vf_tail, vf_end;
  long long live_nodes, live_vars;  // words in use, summed at the end of each turn
  // Scheduler policy (policy.cuh): mode, constant outputs for mode 2 (one
  // triple while fewer redexes than threads are pending, one otherwise; a
  // negative entry keeps the fixed policy's choice), MLP weights for mode 1,
  // and the previous turn's counters for the features.
  unsigned int policy_mode;
  float policy_const[6];
  const float* policy_w;
  unsigned long long prev_itrs, prev_leak, prev_hist[8], turn_t0;
  unsigned int npool_next;          // next page id of the node pool
  unsigned int vpool_next;          // next page id of the var pool
  TurnRecord* trace;                // per-turn records (null = off)
  unsigned int trace_cap;
  unsigned int policy_script_len;   // POLICY_SCRIPT: turns the script covers
  // Persistent launches: the block that closes a turn writes `go` (whether
  // the launch runs another turn) and then raises `epoch`, which the other
  // blocks wait on.
  unsigned int epoch;
  unsigned int go;
  unsigned int persist_ran;         // turns the last persistent launch closed
};

constexpr Pair NODE_MARK = ~(Pair)0;

// Node and var indices below LOCAL_WORDS name a block's local net (shared
// memory) in the local-net kernel variant; the global allocator never hands
// them out (the first pages of each space are reserved in every variant).
constexpr uint32_t LOCAL_WORDS = 2048;
__host__ __device__ __forceinline__ uint32_t reserved_pages(uint32_t page_log2) {
  return (LOCAL_WORDS + (1u << page_log2) - 1) >> page_log2;
}

struct PagedSpace {
  uint32_t page_log2;        // words per page = 1 << page_log2
  uint32_t max_pages;        // capacity of each thread's page list
  uint32_t* lists;           // [nthreads][max_pages] page ids
  uint32_t* counts;          // [nthreads] pages owned
  uint32_t* pos;             // [nthreads] index into the list of the page being scanned
  uint32_t* off;             // [nthreads] word offset of the next chunk in that page
};

// Everything a turn kernel needs; passed by value.
struct Dev {
  Pair* node;                 // node words, 2^k entries
  Port* vars;                 // var words, 2^k entries; var v lives at v & vars_mask,
                              // so ROOT (0x1FFFFFFF) lands on the last word
  uint32_t vars_mask;
  uint32_t node_mask;         // node space size - 1
  Pair* ring;                 // global redex ring
  unsigned long long ring_mask;
  PagedSpace nspace, vspace;  // per-thread page lists (persist across turns)
  uint32_t npool_end, vpool_end;  // one past the last page id the pools may hand out
  uint32_t npool_base, vpool_base;  // first page id of each space the allocator hands out
  uint32_t extra_roots;       // nets in a batch - 1: vars ROOT_VAR - k (k <= extra_roots) are roots
  uint32_t tables;            // 1 when nloc/vloc hold CHUNK words per thread at least
  uint32_t* nfree_ring;       // free-page rings (null: pages are never returned)
  uint32_t* vfree_ring;
  uint32_t nfree_mask, vfree_mask;
  uint32_t* nloc;             // CALL scratch: [max_def_nodes][nthreads]
  uint32_t* vloc;             // CALL scratch: [max_def_vars][nthreads]
  uint32_t nthreads;
  uint32_t ndefs;
  Pair* ovf;                  // local-net variant: OVF_CAP overflow entries per thread
  uint32_t steal_min;         // a lane gives a redex to an empty lane of its warp once it holds this many
  uint32_t rule_select;       // 0: every lane runs its redex each round; 1/2: one rule class / rule per round
  uint32_t fast_calls;        // CALL-time fast paths: 0 off, 1 SWITCH pattern, 2 SWITCH and ANNI
  const DefHdr* defs;
  const Pair* book;
  Ctl* ctl;
#ifdef HVM_COMPILED_CALLS
  uint32_t compiled;          // 1 when the loaded book is the one compiled into this program
#endif
};

// ---- memory access -----------------------------------------------------------

#ifdef HVM_PORT64
// 128-bit node words: one 16-byte access each (a node is seen whole or not
// at all, as the 64-bit words of the 32-bit build are), at gpu scope so that
// no stale L1 line is read. Node indices are masked like var indices.
__device__ __forceinline__ Pair ld_pair(const Pair* p) {
  unsigned long long lo, hi;
  asm volatile("{\n .reg .b128 d;\n ld.relaxed.gpu.global.b128 d, [%2];\n mov.b128 {%0, %1}, d;\n}"
               : "=l"(lo), "=l"(hi) : "l"(p) : "memory");
  return ((Pair)hi << 64) | lo;
}
__device__ __forceinline__ void st_pair(Pair* p, Pair v) {
  asm volatile("{\n .reg .b128 s;\n mov.b128 s, {%1, %2};\n st.relaxed.gpu.global.b128 [%0], s;\n}"
               :: "l"(p), "l"((unsigned long long)v), "l"((unsigned long long)(v >> 64)) : "memory");
}
__device__ __forceinline__ Pair nload(const Dev& d, uint32_t i) { return ld_pair(&d.node[i & d.node_mask]); }
__device__ __forceinline__ void nstore(const Dev& d, uint32_t i, Pair p) { st_pair(&d.node[i & d.node_mask], p); }
// Read-only words (the book): two 64-bit loads through the read-only cache.
__device__ __forceinline__ Pair book_pair(const Pair* p) {
  const unsigned long long* q = (const unsigned long long*)p;
  return ((Pair)__ldg(q + 1) << 64) | __ldg(q);
}
// A redex of the ring, written in an earlier turn.
__device__ __forceinline__ Pair ring_pair(const Pair* p) { return ld_pair(p); }
__device__ __forceinline__ Port vload(const Dev& d, uint32_t i) {
  return (Port)__ldcg((const unsigned long long*)&d.vars[i & d.vars_mask]);
}
__device__ __forceinline__ void vstore(const Dev& d, uint32_t i, Port p) {
  __stcg((unsigned long long*)&d.vars[i & d.vars_mask], (unsigned long long)p);
}
__device__ __forceinline__ Port vexch(const Dev& d, uint32_t i, Port p) {
  return (Port)atomicExch((unsigned long long*)&d.vars[i & d.vars_mask], (unsigned long long)p);
}
#else
__device__ __forceinline__ Pair nload(const Dev& d, uint32_t i) {
  return (Pair)__ldcg((const unsigned long long*)&d.node[i]);
}
__device__ __forceinline__ void nstore(const Dev& d, uint32_t i, Pair p) {
  __stcg((unsigned long long*)&d.node[i], (unsigned long long)p);
}
__device__ __forceinline__ Pair book_pair(const Pair* p) { return (Pair)__ldg((const unsigned long long*)p); }
__device__ __forceinline__ Pair ring_pair(const Pair* p) { return (Pair)__ldcg((const unsigned long long*)p); }
__device__ __forceinline__ Port vload(const Dev& d, uint32_t i) { return __ldcg(&d.vars[i & d.vars_mask]); }
__device__ __forceinline__ void vstore(const Dev& d, uint32_t i, Port p) { __stcg(&d.vars[i & d.vars_mask], p); }
__device__ __forceinline__ Port vexch(const Dev& d, uint32_t i, Port p) { return atomicExch(&d.vars[i & d.vars_mask], p); }
#endif

__device__ __forceinline__ void set_status(const Dev& d, uint32_t code, uint32_t info) {
  if (atomicCAS(&d.ctl->status, 0u, code) == 0u) d.ctl->err_info = info;
}

// Per-thread allocator registers for one space.
struct Alloc {
  uint32_t pos, off, count;  // page-list position, next chunk offset, pages owned
  uint32_t page;             // id of the page at `pos`
  uint32_t chunk;            // word index of the chunk `mask` describes
  uint32_t mask;             // free words of that chunk not yet handed out
  uint32_t dry_chunks;       // chunks scanned since the last free word
  bool pool_dry;             // the page pool ran out during this turn
  bool page_empty;           // every chunk of this page seen in this pass was entirely free
};

// ---- per-thread state ----------------------------------------------------------

struct TState {
  Pair* stk;                  // this thread's deque in shared memory (stride = blockDim.x)
  uint32_t stride;
  uint32_t lo, len, cap;      // entries lo .. lo+len-1 (mod cap); cap is a power of two
  uint32_t gid;
  Alloc na, va;               // node / var allocators
  unsigned long long base;    // ring index of this turn's first input (overflow check)
  uint32_t itrs, leak, retries;  // this turn's counts: budget-bounded, so 32 bits suffice
  int live_nodes, live_vars;  // words taken minus words freed in this turn
  bool dirty;                 // wrote fresh words not yet ordered by a fence
  uint32_t hist[8];
  bool dead;                  // set after a fatal status: stop interacting
  uint32_t waited;            // rounds this lane's next redex has waited for its rule class
};

// ---- local nets (the local-net kernel variant) ----------------------------------
//
// As in the reference's CUDA runtime (src/hvm.cu:130-135, 1129-1174), a
// block's fresh nodes and vars live in shared memory while a turn runs, and
// nothing in global memory may point into it: indices below LOCAL_WORDS name
// the block's local words. A lane owns a slice of LOCAL_SLICE nodes and vars.
// The linker never writes a local port into a global var (it redirects a
// local var, and turns a local node into a LEAK redex that copies it out);
// a fresh global node never holds a local port; redexes that name local
// words stay with the lane (its deque, and an overflow stack of its own in
// global memory) until the turn's end, when every one of them is made
// global -- its local ends wired to fresh global vars, its local nodes
// copied out by LEAK -- before the flush to the ring.
constexpr uint32_t LOCAL_SLICE = 16;      // local nodes and vars per lane (128-thread blocks)
constexpr uint32_t OVF_CAP = 256;         // a lane's overflow stack
constexpr uint32_t OVF_HIGH = OVF_CAP - 64;  // a warp whose lane holds more ends its turn
__device__ __forceinline__ bool is_local(Port p) {
  return (get_tag(p) == VAR || get_tag(p) >= CON) && get_val(p) < LOCAL_WORDS && p != 0;
}
__device__ __forceinline__ bool is_gvar(Port p) { return get_tag(p) == VAR && get_val(p) >= LOCAL_WORDS; }
__device__ __forceinline__ bool local_pair(Pair r) { return is_local(get_fst(r)) || is_local(get_snd(r)); }

// The local-net variant's per-block arrays follow the deques in dynamic
// shared memory: local nodes, local vars, then each lane's overflow length;
// a lane's slice starts at threadIdx.x * LOCAL_SLICE, and its overflow stack
// (global memory, read and written by that lane only) at gid * OVF_CAP. They
// are computed rather than kept in the thread state, which the default
// variants share.
__device__ __forceinline__ Pair* lnode_of(const TState& t) { return t.stk - threadIdx.x + (size_t)t.stride * t.cap; }
__device__ __forceinline__ Port* lvar_of(const TState& t) { return (Port*)(lnode_of(t) + LOCAL_WORDS); }
__device__ __forceinline__ uint32_t& ovf_len_of(const TState& t) { return ((uint32_t*)(lvar_of(t) + LOCAL_WORDS))[threadIdx.x]; }
__device__ __forceinline__ Pair* ovf_of(const Dev& d, const TState& t) { return d.ovf + (size_t)t.gid * OVF_CAP; }
__device__ __forceinline__ uint32_t lbase_of() { return threadIdx.x * LOCAL_SLICE; }

// Net word access that resolves local indices to the block's shared arrays.
template <bool LOCAL>
__device__ __forceinline__ Pair n_load(const Dev& d, const TState& t, uint32_t i) {
  if (LOCAL && i < LOCAL_WORDS) return ((volatile Pair*)lnode_of(t))[i];
  return nload(d, i);
}
template <bool LOCAL>
__device__ __forceinline__ void n_store(const Dev& d, const TState& t, uint32_t i, Pair p) {
  if (LOCAL && i < LOCAL_WORDS) ((volatile Pair*)lnode_of(t))[i] = p;
  else nstore(d, i, p);
}
template <bool LOCAL>
__device__ __forceinline__ void v_store(const Dev& d, const TState& t, uint32_t i, Port p) {
  if (LOCAL && i < LOCAL_WORDS) ((volatile Port*)lvar_of(t))[i] = p;
  else vstore(d, i, p);
}
template <bool LOCAL>
__device__ __forceinline__ Port v_exch(const Dev& d, const TState& t, uint32_t i, Port p) {
  if (LOCAL && i < LOCAL_WORDS) {
#ifdef HVM_PORT64
    return (Port)atomicExch((unsigned long long*)&lvar_of(t)[i], (unsigned long long)p);
#else
    return atomicExch(&lvar_of(t)[i], p);
#endif
  }
  return vexch(d, i, p);
}
// Live-word accounting counts global words only (local ones end with the turn).
__device__ __forceinline__ int global_words(uint32_t i, int n) { return i < LOCAL_WORDS ? 0 : n; }

// Rule classes for per-round selection: mode 1 groups the rules by the code
// they run -- no allocation (LINK, VOID, ERAS, ANNI), CALL, COMM, one or two
// fresh nodes (OPER, SWIT); mode 2 uses the rule itself. Only a scheduling
// choice: plan_redex still decides what the interaction is.
constexpr uint32_t RULE_WAIT_MAX = 4;  // rounds a lane may wait before its class goes first
__device__ __forceinline__ uint32_t rule_class(uint32_t mode, Pair r) {
  const Rule rule = get_rule(get_fst(r), get_snd(r));
  if (mode == 2) return rule;
  if (rule == CALL) return 1;
  if (rule == COMM) return 2;
  if (rule == OPER || rule == SWIT) return 3;
  return 0;
}

// Local redex deque: the thread pops and pushes at the top (LIFO, depth
// first, like the reference's per-thread bags); when it is full, the oldest
// half moves to the global ring with one atomic (those are the redexes other
// threads will take first next turn).
__device__ __forceinline__ Pair& slot(TState& t, uint32_t i) {
  return t.stk[(size_t)((t.lo + i) & (t.cap - 1)) * t.stride];
}

template <bool LOCAL = false>
__device__ __forceinline__ void spill_oldest(const Dev& d, TState& t, uint32_t k) {
  if constexpr (LOCAL) {
    // Local-net variant: the spilled redexes may name local words, so they
    // stay with the lane; a warp ends its turn before an overflow fills.
    uint32_t& n = ovf_len_of(t);
    if (n + k > OVF_CAP) { set_status(d, ST_RING_FULL, 2); t.dead = true; return; }
    for (uint32_t i = 0; i < k; i++) ovf_of(d, t)[n + i] = slot(t, i);
    n += k;
    t.lo = (t.lo + k) & (t.cap - 1);
    t.len -= k;
    return;
  }
  unsigned long long at = atomicAdd(&d.ctl->tail, (unsigned long long)k);
  if (at + k - t.base > d.ring_mask + 1) { set_status(d, ST_RING_FULL, 0); t.dead = true; return; }
  for (uint32_t i = 0; i < k; i++) d.ring[(at + i) & d.ring_mask] = slot(t, i);
  t.lo = (t.lo + k) & (t.cap - 1);
  t.len -= k;
  t.leak += k;
}

template <bool LOCAL = false>
__device__ __forceinline__ void push(const Dev& d, TState& t, Pair r) {
  if (t.len == t.cap) {
    spill_oldest<LOCAL>(d, t, t.cap / 2);
    if (t.dead) return;
  }
  slot(t, t.len) = r;
  t.len++;
}

__device__ __forceinline__ Pair pop(TState& t) {
  t.len--;
  return slot(t, t.len);
}

// ---- allocation (src/hvm.cu:880-912, src/hvm.c:713-755) ------------------------
//
// As in the reference, a thread allocates by scanning memory it owns for free
// (zero) words with a cursor that persists across turns, so words freed by
// any thread are reused when the cursor comes back round. The GB300 layout:
//   * the node and var spaces are cut into pages (a power of two of words,
//     >= one 64-byte chunk); each thread owns a list of pages exclusively, so
//     a word it sees free stays free until it takes it -- no atomics;
//   * the scan reads one 64-byte chunk per L2 round trip (8 node words or 16
//     var words, vector loads) and keeps a bitmask of the free words, so most
//     allocations cost no memory access at all;
//   * a thread that scanned two pages' worth of chunks without finding a free
//     word takes a fresh page from a global pool (one atomic) instead of
//     failing; only an exhausted pool or page list is out-of-memory.
// A node word is marked (all ones) as soon as it is taken, so a later scan
// of the same chunk inside one interaction cannot hand it out twice; the
// last node word is never used, so the mark is not a real node. A var is
// created (NONE) as soon as it is taken. Word 0 of each space and the ROOT
// var (the last var word) are never handed out.

__device__ __forceinline__ unsigned int* pool_counter(const Dev& d, bool vars) {
  return vars ? &d.ctl->vpool_next : &d.ctl->npool_next;
}

// 256-bit load that bypasses L1 (sm_100+).
__device__ __forceinline__ void ld_cg_v4(const void* p, unsigned long long& a, unsigned long long& b,
                                         unsigned long long& c, unsigned long long& e) {
  asm volatile("ld.global.cg.v4.u64 {%0,%1,%2,%3}, [%4];" : "=l"(a), "=l"(b), "=l"(c), "=l"(e) : "l"(p));
}

constexpr uint32_t CHUNK = 32;  // words per scanned chunk (256 B of nodes, 128 B of vars)
constexpr uint32_t MAX_DRY_PAGES = 4;  // full cycles over a lane's pages before out-of-memory
constexpr uint32_t SOFT_RUN_CHUNKS = 64;  // chunks a CALL scans for a contiguous run before taking single words
constexpr uint32_t SOFT_GRAB_PAGES = 8;   // a contiguous-run request may take pages up to this many owned

// Bit i of the result is set when word base+i is free and may be handed out.
template <bool VARS>
__device__ __forceinline__ uint32_t chunk_mask(const Dev& d, uint32_t base) {
  uint32_t m = 0;
  if (!VARS) {
#ifdef HVM_PORT64
    #pragma unroll
    for (int k = 0; k < 16; k++) {  // two 16-byte nodes per 32-byte load
      unsigned long long w0, w1, w2, w3;
      ld_cg_v4(&d.node[base + 2 * k], w0, w1, w2, w3);
      m |= ((w0 == 0 && w1 == 0) | (w2 == 0 && w3 == 0) << 1) << (2 * k);
    }
#else
    #pragma unroll
    for (int k = 0; k < 8; k++) {
      unsigned long long w0, w1, w2, w3;
      ld_cg_v4(&d.node[base + 4 * k], w0, w1, w2, w3);
      m |= ((w0 == 0) | (w1 == 0) << 1 | (w2 == 0) << 2 | (w3 == 0) << 3) << (4 * k);
    }
#endif
    if ((uint64_t)base + CHUNK > d.node_mask) m &= ~(1u << (d.node_mask - base));  // never the MARK word
  } else {
#ifdef HVM_PORT64
    #pragma unroll
    for (int k = 0; k < 8; k++) {  // four 8-byte vars per 32-byte load
      unsigned long long w0, w1, w2, w3;
      ld_cg_v4(&d.vars[base + 4 * k], w0, w1, w2, w3);
      m |= ((w0 == 0) | (w1 == 0) << 1 | (w2 == 0) << 2 | (w3 == 0) << 3) << (4 * k);
    }
#else
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      unsigned long long w0, w1, w2, w3;
      ld_cg_v4(&d.vars[base + 8 * k], w0, w1, w2, w3);
      uint32_t b8 = 0;
      b8 |= ((uint32_t)w0 == 0) | ((uint32_t)(w0 >> 32) == 0) << 1;
      b8 |= ((uint32_t)w1 == 0) << 2 | ((uint32_t)(w1 >> 32) == 0) << 3;
      b8 |= ((uint32_t)w2 == 0) << 4 | ((uint32_t)(w2 >> 32) == 0) << 5;
      b8 |= ((uint32_t)w3 == 0) << 6 | ((uint32_t)(w3 >> 32) == 0) << 7;
      m |= b8 << (8 * k);
    }
#endif
    if ((uint64_t)base + CHUNK > d.vars_mask) m &= ~(1u << (d.vars_mask - base));  // ROOT
  }
  if (base == 0) m &= ~1u;
  return m;
}

// Bit i set iff bits i .. i+n-1 of m are all set (1 <= n <= 32).
__device__ __forceinline__ uint32_t runs_of(uint32_t m, uint32_t n) {
  uint32_t len = 1;
  while (len * 2 <= n) { m &= m >> len; len <<= 1; }
  if (len < n) m &= m >> (n - len);
  return m;
}

// Takes n (1..32) consecutive free words of one chunk; returns the first, or
// 0 when the page list is full and the pool is empty. Taken words are
// written at once (vars as NONE, nodes as MARK) so no later scan can see them
// free before their owner fills them.
template <bool VARS, bool MARK = true>
__device__ __forceinline__ uint32_t alloc_run(const Dev& d, TState& t, Alloc& a, uint32_t n, uint32_t soft_limit = 0) {
  const PagedSpace& sp = VARS ? d.vspace : d.nspace;
  const uint32_t page_words = 1u << sp.page_log2;
  const uint32_t chunks_per_page = page_words / CHUNK;
  uint32_t scanned = 0;
  for (uint32_t guard = 0; guard < (1u << 22); guard++) {
    uint32_t r = runs_of(a.mask, n);
    if (r) {
      uint32_t b = __ffs(r) - 1;
      a.mask &= ~((n == 32 ? ~0u : (1u << n) - 1) << b);
      uint32_t at = a.chunk + b;
      for (uint32_t i = 0; i < n; i++) {
        if (VARS) vstore(d, at + i, NONE);
        else if (MARK) nstore(d, at + i, NODE_MARK);
      }
      if (VARS) t.live_vars += n; else t.live_nodes += n;
      return at;
    }
    // Leaving a chunk that was entirely free and untouched keeps the page a
    // candidate for return.
    if (a.mask != 0xFFFFFFFFu) a.page_empty = false;
    // Next chunk: within the page, then the next owned page, then a new page.
    if (a.off >= page_words) {
      a.off = 0;
      uint32_t* ring = VARS ? d.vfree_ring : d.nfree_ring;
      bool moved = false;
      if (a.page_empty && a.count > 1 && ring) {
        // The whole page is free: give it back to the free-page ring and
        // drop it from this lane's list.
        unsigned int* tail = VARS ? &d.ctl->vf_tail : &d.ctl->nf_tail;
        ring[atomicAdd(tail, 1u) & (VARS ? d.vfree_mask : d.nfree_mask)] = a.page;
        uint32_t* list = sp.lists + (size_t)t.gid * sp.max_pages;
        list[a.pos] = list[a.count - 1];
        a.count--;
        sp.counts[t.gid] = a.count;
        if (a.pos >= a.count) a.pos = 0;
        a.page = list[a.pos];
        a.page_empty = true;
        moved = true;  // scan the page that took its place
      }
      bool grabbed = moved;
      // A soft request (a contiguous run) takes a page only while the lane
      // owns few, so pages are not hoarded for fragmentation alone.
      if (!moved && (!soft_limit || a.count < SOFT_GRAB_PAGES) && (a.dry_chunks >= 2 * chunks_per_page || (a.count == 1 && a.dry_chunks >= chunks_per_page)) &&
          a.count < sp.max_pages && !a.pool_dry) {
        uint32_t fresh = 0xFFFFFFFFu;
        if (ring) {  // a returned page first
          unsigned int* head = VARS ? &d.ctl->vf_head : &d.ctl->nf_head;
          unsigned int end = __ldcg(VARS ? &d.ctl->vf_end : &d.ctl->nf_end);
          if (__ldcg(head) < end) {
            unsigned int h = atomicAdd(head, 1u);
            if (h < end) fresh = __ldcg(&ring[h & (VARS ? d.vfree_mask : d.nfree_mask)]);
          }
        }
        if (fresh == 0xFFFFFFFFu) {
          uint32_t f = atomicAdd(pool_counter(d, VARS), 1u);
          if (f < (VARS ? d.vpool_end : d.npool_end)) fresh = f;
        }
        if (fresh != 0xFFFFFFFFu) {
          sp.lists[(size_t)t.gid * sp.max_pages + a.count] = fresh;
          a.pos = a.count;
          a.count++;
          sp.counts[t.gid] = a.count;
          a.page = fresh;
          a.dry_chunks = 0;
          a.page_empty = true;
          grabbed = true;
        } else {
          a.pool_dry = true;  // no page anywhere: keep cycling through owned pages
        }
      }
      if (!grabbed) {
        // Every owned page scanned several times over without room: full.
        if (a.dry_chunks >= MAX_DRY_PAGES * chunks_per_page * a.count) {
          if (atomicCAS(&d.ctl->oom_space, 0u, VARS ? 2u : 1u) == 0u) {
            d.ctl->oom_pages = a.count;
            d.ctl->oom_dry = a.dry_chunks;
            d.ctl->oom_pool_dry = a.pool_dry ? 1u : 0u;
          }
          return 0;
        }
        a.pos = a.pos + 1 == a.count ? 0 : a.pos + 1;
        a.page = __ldcg(&sp.lists[(size_t)t.gid * sp.max_pages + a.pos]);
        a.page_empty = true;
      }
    }
    // A soft request (a contiguous run the caller can do without) gives up
    // after `soft_limit` chunks instead of growing or failing.
    if (soft_limit && scanned++ >= soft_limit) return 0;
    a.chunk = (a.page << sp.page_log2) + a.off;
    a.off += CHUNK;
    a.mask = chunk_mask<VARS>(d, a.chunk);
    a.dry_chunks = runs_of(a.mask, n) ? 0 : a.dry_chunks + 1;
  }
  return 0;
}

__device__ __forceinline__ uint32_t alloc_node(const Dev& d, TState& t) { return alloc_run<false>(d, t, t.na, 1); }

// Local-net variant: n (<= LOCAL_SLICE) consecutive free words of the lane's
// slice of the block's local net, or 0. The slice's words are read afresh
// (other lanes free words in it when they take them); taken vars are created
// (NONE) at once, taken nodes are written by the caller before the lane's
// next allocation.
template <bool VARS>
__device__ __forceinline__ uint32_t lalloc(TState& t, uint32_t n) {
  uint32_t m = 0;
  if (VARS) {
    const unsigned at = (unsigned)__cvta_generic_to_shared(lvar_of(t) + lbase_of());
    #pragma unroll
    for (int k = 0; k < (int)LOCAL_SLICE / 4; k++) {
      unsigned x, y, z, w;
      asm volatile("ld.shared.v4.u32 {%0,%1,%2,%3}, [%4];" : "=r"(x), "=r"(y), "=r"(z), "=r"(w) : "r"(at + 16 * k) : "memory");
      m |= ((x == 0) | (y == 0) << 1 | (z == 0) << 2 | (w == 0) << 3) << (4 * k);
    }
  } else {
    const unsigned at = (unsigned)__cvta_generic_to_shared(lnode_of(t) + lbase_of());
    #pragma unroll
    for (int k = 0; k < (int)LOCAL_SLICE / 2; k++) {
      unsigned long long x, y;
      asm volatile("ld.shared.v2.u64 {%0,%1}, [%2];" : "=l"(x), "=l"(y) : "r"(at + 16 * k) : "memory");
      m |= ((x == 0) | (y == 0) << 1) << (2 * k);
    }
  }
  if (threadIdx.x == 0) m &= ~1u;  // index 0 is never handed out
  const uint32_t r = runs_of(m, n);
  if (!r) return 0;
  const uint32_t at = lbase_of() + (__ffs(r) - 1);
  if (VARS)
    for (uint32_t i = 0; i < n; i++) ((volatile Port*)lvar_of(t))[at + i] = NONE;
  return at;
}
__device__ __forceinline__ uint32_t alloc_var(const Dev& d, TState& t) { return alloc_run<true>(d, t, t.va, 1); }

// Loads a thread's allocator state at turn start; it resumes at the chunk it
// was scanning when the previous turn ended.
template <bool VARS>
__device__ __forceinline__ void alloc_load(const PagedSpace& sp, uint32_t gid, Alloc& a) {
  const uint32_t chunk_words = CHUNK;
  a.pos = sp.pos[gid];
  a.off = sp.off[gid];
  a.count = sp.counts[gid];
  a.page = sp.lists[(size_t)gid * sp.max_pages + a.pos];
  a.off = a.off >= chunk_words ? a.off - chunk_words : 0;
  a.chunk = 0;
  a.mask = 0;
  a.dry_chunks = 0;
  a.pool_dry = false;
  a.page_empty = false;  // resumed mid-page: unknown
}

__device__ __forceinline__ void alloc_save(const PagedSpace& sp, uint32_t gid, const Alloc& a) {
  sp.pos[gid] = a.pos;
  sp.off[gid] = a.off;
}

// ---- warp-lockstep interactions (src/hvm.c:784-1122) -----------------------------
//
// Every lane of a warp runs one interaction per round, and all lanes walk the
// same phases in the same order, whatever their rule:
//   1. plan    -- rule, swap, def header (no memory traffic beyond the book);
//   2. load    -- the principal nodes (one predicated load each, all lanes);
//   3. alloc   -- fresh node/var words from the lane's chunk masks;
//   4. write   -- take the principal nodes, create the new nodes;
//   5. fence   -- one gpu-scope fence for the warp, before anything created
//                 can be reached by another thread through a link;
//   6. link    -- the rule's list of port pairs, wired by the reference's
//                 lock-free linker (src/hvm.c:793-840) one step per round:
//                 each step is a single atomic exchange issued by every
//                 active lane together.
// The reference runs the same rules with a divergent switch per thread,
// which on a SIMT machine serialises the memory round trips of the
// different rules; here a warp pays about one round trip per phase.

enum : int { IR_DONE = 0, IR_RETRY = 1, IR_FATAL = 2 };

// Profile counters (per warp, lane 0, summed into Ctl::prof when enabled).
enum { PROF_ROUNDS, PROF_LANES, PROF_STEPS, PROF_CYC_ROUND, PROF_CYC_LOAD, PROF_CYC_WRITE, PROF_CYC_FENCE, PROF_CYC_LINK };
struct WarpProf { unsigned long long v[8]; };

// What one lane does this round.
struct Plan {
  Port a, b;            // ports after the swap (src/hvm.c:1090-1097)
  Pair A, B;            // principal nodes of a and b (when the rule takes them)
  uint32_t rule;        // LINK..SWIT; IDLE_RULE for a lane without a redex
  uint32_t nlinks;      // port pairs to wire
  // COMM/OPER/SWIT take their fresh nodes (and COMM its vars) as one run each,
  // at nbase + k and vbase + k.
  uint32_t node_len, rbag_len, vars_len, off;  // CALL: the def
  uint32_t nbase, vbase;  // CALL: first fresh node / var (contiguous runs), or
  bool contig;            //       per-word scratch tables when the def is large
  bool joined;            // CALL: the def's links include the root link (DefHdr::joined)
  Port root;            // CALL: the def's root
  Numb cv;              // OPER: the result when both sides are numbers
  bool oper_num;        // OPER: B1 is a number
  bool counted;         // counts as an interaction (every rule but LINK)
  uint32_t fpad;        // CALL: the def's fast-path word (0 unless the caller is a CON)
  uint32_t fast;        // CALL: 0, or the fast path taken: 1 ANNI, 2 SWITCH on 0, 3 SWITCH on X > 0
  Port f1, f2;          // CALL fast path: the def-side ports of its two links
  Port lx1, ly1, lx2, ly2;  // local-net variant: extra links of LEAK, GLOBALIZE and a fresh global
                            // node's fixed-up port
#ifdef HVM_COMPILED_CALLS
  uint32_t fid;         // CALL: the def
#endif
};
constexpr uint32_t IDLE_RULE = 8;
// Local-net variant only: LEAK copies a local node out to a global var's
// target (src/hvm.cu:1129-1174); GLOBALIZE, at a turn's end, wires a redex's
// local ends to fresh global vars so the redex can go to the ring. Neither
// counts as an interaction.
constexpr uint32_t LEAK_RULE = 9, GLOB_RULE = 10;

#ifdef HVM_COMPILED_CALLS
// Compiled calls (the reference's compile_book for its CUDA target,
// src/cmp.rs:10-119, which src/main.rs:140-146 leaves disabled): a program
// emitted by `hvm gen-cu --compiled` defines these from its book, as
// straight-line code per def, with the def's words as immediates instead of
// loads from the def tables. Both are used for contiguous runs only, and
// both return false for a def that was not compiled (it then runs from the
// tables); the interactions are the same either way.
// Writes def fid's nodes at nb, nb+1, ... (their vars at vb, vb+1, ...).
__device__ __forceinline__ bool compiled_call_nodes(const Dev& d, uint32_t fid, uint32_t nb, uint32_t vb);
// The i-th link of def fid (its redexes, then its root ~ `caller`).
__device__ __forceinline__ bool compiled_call_link(uint32_t fid, uint32_t i, uint32_t nb, uint32_t vb, Port caller,
                                                   Port& x, Port& y);
#endif

// Maps a def-local port to the fresh words of this CALL (adjust_port,
// src/hvm.c:346-362): base + index for contiguous runs, else the scratch tables.
__device__ __forceinline__ Port relocate(const Dev& d, uint32_t gid, const Plan& pl, Port p) {
  Tag tag = get_tag(p);
  if (pl.contig) {
    if (tag >= CON) return new_port(tag, pl.nbase + get_val(p));
    if (tag == VAR) return new_port(VAR, pl.vbase + get_val(p));
    return p;
  }
  if (tag >= CON) return new_port(tag, d.nloc[(size_t)get_val(p) * d.nthreads + gid]);
  if (tag == VAR) return new_port(VAR, d.vloc[(size_t)get_val(p) * d.nthreads + gid]);
  return p;
}

// The i-th port pair of the lane's rule (src/hvm.c:852-1070).
template <bool FAST, bool LOCAL>
__device__ __forceinline__ void link_pair(const Dev& d, uint32_t gid, const Plan& p, uint32_t i, Port& x, Port& y) {
  if (LOCAL && (p.rule == LEAK_RULE || p.rule == GLOB_RULE || ((p.rule == OPER || p.rule == SWIT) && i > 0))) {
    // LEAK: the global var ~ the copied node, then its children's wires;
    // GLOBALIZE: its wires; OPER/SWIT: link 1 is the fixed-up port's wire.
    const uint32_t j = p.rule == LEAK_RULE ? i : p.rule == GLOB_RULE ? i + 1 : i;
    if (j == 0) { x = p.a; y = new_port(get_tag(p.b), p.nbase); }
    else if (j == 1) { x = p.lx1; y = p.ly1; }
    else { x = p.lx2; y = p.ly2; }
    return;
  }
  switch (p.rule) {
    case LINK: x = p.a; y = p.b; break;
    case ERAS: x = p.a; y = i == 0 ? get_fst(p.B) : get_snd(p.B); break;
    case ANNI:
      x = i == 0 ? get_fst(p.A) : get_snd(p.A);
      y = i == 0 ? get_fst(p.B) : get_snd(p.B);
      break;
    case COMM: {
      x = new_port(i < 2 ? get_tag(p.b) : get_tag(p.a), p.nbase + i);
      y = i == 0 ? get_fst(p.A) : i == 1 ? get_snd(p.A) : i == 2 ? get_fst(p.B) : get_snd(p.B);
      break;
    }
    case OPER:
      if (p.oper_num) { x = new_port(NUM, p.cv); y = get_snd(p.B); }
      else { x = get_fst(p.B); y = new_port(OPR, p.nbase); }
      break;
    case SWIT: x = new_port(CON, p.nbase); y = get_fst(p.B); break;
    default: {  // CALL
      if (FAST && p.fast && i + 1 >= p.rbag_len) {
        // The root link (the last one) becomes the fast path's two links
        // (src/cmp.rs:120-245): ANNI root ~ (B1 B2): r1 ~ B1, r2 ~ B2;
        // SWITCH on 0: s1 ~ R, s2 ~ *; on X > 0: s1 ~ *, s2 ~ b = (#(X-1) R).
        const bool second = i + 1 > p.rbag_len;
        x = relocate(d, gid, p, second ? p.f2 : p.f1);
        if (p.fast == 1) y = second ? get_snd(p.B) : get_fst(p.B);
        else if (p.fast == 2) y = second ? new_port(ERA, 0) : get_snd(p.B);
        else y = second ? new_port(CON, get_val(p.b)) : new_port(ERA, 0);
        break;
      }
#ifdef HVM_COMPILED_CALLS
      if (d.compiled && p.contig && compiled_call_link(p.fid, i, p.nbase, p.vbase, p.b, x, y)) break;
#endif
      if (i < p.rbag_len) {
        Pair q = book_pair(&d.book[p.off + i]);
        x = get_fst(q) == CALLER_PORT ? p.b : relocate(d, gid, p, get_fst(q));
        y = get_snd(q) == CALLER_PORT ? p.b : relocate(d, gid, p, get_snd(q));
      } else {
        x = relocate(d, gid, p, p.root);
        y = p.b;
      }
      break;
    }
  }
}

// Plans lane's interaction on redex r; returns false for an invalid REF.
template <bool FAST, bool LOCAL>
__device__ __forceinline__ bool plan_redex(const Dev& d, TState& t, Pair r, Plan& p, bool drain) {
  Port a = get_fst(r), b = get_snd(r);
  uint32_t rule = get_rule(a, b);
  // REF ~ ROOT is a call (src/hvm.c:1090-1092); a batch has one ROOT var per net.
  if (get_tag(a) == REF && get_tag(b) == VAR && get_val(b) >= ROOT_VAR - d.extra_roots) rule = CALL;
  else if (should_swap(a, b)) { Port x = a; a = b; b = x; }
  p.a = a; p.b = b;
  if (LOCAL) {
    // A global var meeting a local node is a LEAK; at a turn's end every
    // other redex that names local words is made global.
    if (rule == LINK && is_gvar(a) && get_tag(b) >= CON && get_val(b) < LOCAL_WORDS) rule = LEAK_RULE;
    else if (drain) rule = GLOB_RULE;
  }
  if constexpr (LOCAL) p.counted = rule != LINK && rule != LEAK_RULE && rule != GLOB_RULE;
  else p.counted = rule != LINK;
  p.node_len = p.rbag_len = p.vars_len = 0;
  p.fpad = 0;
  p.fast = 0;
  if (rule == CALL) {
    uint32_t fid = get_val(a) & 0xFFFFFFFu;
    if (fid >= d.ndefs) { set_status(d, ST_BAD_REF, fid); t.dead = true; return false; }
    const DefHdr h = d.defs[fid];
    if (h.safe && get_tag(b) == DUP) {
      rule = ERAS;  // copy optimisation (src/hvm.c:870-873): still one interaction
    } else {
      p.node_len = h.node_len; p.rbag_len = h.rbag_len; p.vars_len = h.vars_len;
      p.off = h.off; p.root = h.root; p.joined = h.joined != 0;
      // CALL-time fast paths, as configured: 1 the SWITCH pattern only, 2 also ANNI.
      if (FAST && d.fast_calls && get_tag(b) == CON && (d.fast_calls >= 2 || fast_kind(h.fast) == FAST_SWITCH))
        p.fpad = h.fast;
#ifdef HVM_COMPILED_CALLS
      p.fid = fid;
      if (d.compiled) p.fpad = 0;  // compiled calls write every node of the def
#endif
    }
  }
  p.rule = rule;
  return true;
}

// One in-flight link A ~ B of the reference's linker (src/hvm.c:811-840),
// advanced one exchange at a time.
struct Slot {
  Port X, Y;
  bool busy, entered;
};

// Takes the lane's next port pairs into an idle slot, wiring on the spot every
// pair that needs no exchange (both sides principal: a new redex).
template <bool FAST, bool LOCAL>
__device__ __forceinline__ void slot_fill(const Dev& d, TState& t, const Plan& p, uint32_t& next, Slot& s) {
  while (!s.busy && next < p.nlinks) {
    link_pair<FAST, LOCAL>(d, t.gid, p, next++, s.X, s.Y);
    if (get_tag(s.X) != VAR && get_tag(s.Y) == VAR) { Port z = s.X; s.X = s.Y; s.Y = z; }
    if (get_tag(s.X) != VAR) push<LOCAL>(d, t, new_pair(s.X, s.Y));
    else { s.busy = true; s.entered = false; }
  }
}

// The exchange this slot needs next: enter Y while it is a var
// (src/hvm.c:793-808), then publish X -> Y.
// Local-net variant, before a slot's next step: a global var may not be
// pointed at a local word. A local var is swapped in as the side written (it
// then points at the global var, entered first); a local node becomes a LEAK
// redex that copies it out (src/hvm.cu:1049-1079).
template <bool LOCAL>
__device__ __forceinline__ void slot_leak(const Dev& d, TState& t, Slot& s) {
  if (!LOCAL || !s.busy) return;
  const bool enter_step = !s.entered && get_tag(s.Y) == VAR;
  if (enter_step || !is_gvar(s.X) || !is_local(s.Y)) return;
  if (get_tag(s.Y) == VAR) {
    Port z = s.X; s.X = s.Y; s.Y = z;
    s.entered = false;
  } else {
    push<LOCAL>(d, t, new_pair(s.X, s.Y));
    s.busy = false;
  }
}

__device__ __forceinline__ void slot_request(const Slot& s, uint32_t& addr, Port& put) {
  const bool enter_step = !s.entered && get_tag(s.Y) == VAR;
  addr = enter_step ? get_val(s.Y) : get_val(s.X);
  put = enter_step ? NONE : s.Y;
}

template <bool LOCAL>
__device__ __forceinline__ void slot_result(const Dev& d, TState& t, Slot& s, uint32_t addr, Port got) {
  if (!s.busy) return;
  const bool enter_step = !s.entered && get_tag(s.Y) == VAR;
  if (enter_step) {
    if (got == NONE || got == 0) s.entered = true;
    else {
      if constexpr (LOCAL) { v_store<LOCAL>(d, t, addr, 0); t.live_vars -= global_words(addr, 1); }
      else { vstore(d, addr, 0); t.live_vars--; }
      s.Y = got;
    }
  } else if (got == NONE) {
    s.busy = false;  // the other side will find Y here
  } else if (got == 0) {
    set_status(d, ST_LINK_UNSET, addr); t.dead = true; s.busy = false;
  } else {
    // The other side had published `got` for X: take X and wire got ~ Y.
    if constexpr (LOCAL) { v_store<LOCAL>(d, t, addr, 0); t.live_vars -= global_words(addr, 1); }
    else { vstore(d, addr, 0); t.live_vars--; }
    s.X = got;
    s.entered = false;
    if (get_tag(s.X) != VAR && get_tag(s.Y) == VAR) { Port z = s.X; s.X = s.Y; s.Y = z; }
    if (get_tag(s.X) != VAR) { push<LOCAL>(d, t, new_pair(s.X, s.Y)); s.busy = false; }
  }
}

// Runs one round for the warp: every lane with `has` interacts on `r`.
// Returns the lane's outcome (IR_DONE / IR_RETRY / IR_FATAL).
// Local-net variant: a redex made global at a turn's end goes to the ring.
__device__ __forceinline__ void ring_put(const Dev& d, TState& t, Pair r) {
  const unsigned long long at = atomicAdd(&d.ctl->tail, 1ull);
  if (at + 1 - t.base > d.ring_mask + 1) { set_status(d, ST_RING_FULL, 3); t.dead = true; return; }
  d.ring[at & d.ring_mask] = r;
  t.leak++;
}

// `drain` (local-net variant, at a turn's end): every redex given is made
// global (LEAK or GLOBALIZE) instead of interacting. HREG selects how the
// per-rule counters are indexed: by constant indices (the thread state then
// lives in registers), or by the rule (which keeps the thread state in local
// memory) -- measured faster for the 64-register variant, whose registers
// cannot hold the state. (Per-block counters in shared memory, added once per
// warp round, measured slower than either.)
template <bool FAST, bool LOCAL, bool HREG = true>
__device__ __forceinline__ int lockstep_round(const Dev& d, TState& t, bool has, Pair r, WarpProf* wp,
                                              bool drain = false) {
  long long c0 = wp ? clock64() : 0;
  Plan p;
  p.rule = IDLE_RULE;
  p.nlinks = 0;
  p.A = p.B = 0;
  if (has && !plan_redex<FAST, LOCAL>(d, t, r, p, LOCAL && drain)) has = false;
  const uint32_t rule = p.rule;

  // 2. load the principal nodes
  const bool needA = rule == ANNI || rule == COMM;
  const bool needB = rule == ERAS || rule == ANNI || rule == COMM || rule == OPER || rule == SWIT ||
                     (LOCAL && rule == LEAK_RULE);
  const bool peekB = FAST && rule == CALL && fast_kind(p.fpad);  // a CALL fast path needs the caller's node
  if (needA) p.A = n_load<LOCAL>(d, t, get_val(p.a));
  if (needB || peekB) p.B = n_load<LOCAL>(d, t, get_val(p.b));
  int rc = IR_DONE;
  if ((needA && p.A == 0) || (needB && p.B == 0)) rc = IR_RETRY;  // not yet visible: re-try later
  if (peekB && p.B != 0) {
    // Fast SWITCH when the caller's first port is a number, else fast ANNI.
    const bool sw = fast_kind(p.fpad) == FAST_SWITCH && get_tag(get_fst(p.B)) == NUM;
    p.fast = sw ? (get_u24(get_val(get_fst(p.B))) == 0 ? 2u : 3u) : d.fast_calls >= 2 ? 1u : 0u;
    if (p.fast) {
      const Pair q = book_pair(&d.book[p.off + p.rbag_len + p.node_len + (sw ? 1 : 0)]);
      p.f1 = get_fst(q);
      p.f2 = get_snd(q);
    }
  }
  long long c1 = 0;
  if (wp) { __syncwarp(); c1 = clock64(); }

  // 3. allocate; 4. write
  bool made = false;
  if (rc == IR_DONE && rule != IDLE_RULE) {
    if (needA) n_store<LOCAL>(d, t, get_val(p.a), 0);
    if (needB) n_store<LOCAL>(d, t, get_val(p.b), 0);
    if (LOCAL) t.live_nodes -= (needA ? global_words(get_val(p.a), 1) : 0) + (needB ? global_words(get_val(p.b), 1) : 0);
    else t.live_nodes -= (needA ? 1 : 0) + (needB ? 1 : 0);
    if constexpr (LOCAL) {
      if (rule == LEAK_RULE) {
        // a (a global var) ~ b (a local node, taken above): copy the node to
        // a fresh global node whose local children become fresh global vars
        // wired to them, and point a at the copy (src/hvm.cu:1136-1174).
        const Port c1 = get_fst(p.B), c2 = get_snd(p.B);
        const bool l1 = is_local(c1), l2 = is_local(c2);
        p.nbase = alloc_run<false, false>(d, t, t.na, 1);
        const uint32_t g1 = l1 ? alloc_run<true>(d, t, t.va, 1) : 1;
        const uint32_t g2 = l2 ? alloc_run<true>(d, t, t.va, 1) : 1;
        if (!p.nbase || !g1 || !g2) {
          rc = IR_FATAL;
        } else {
          const Port n1 = l1 ? new_port(VAR, g1) : c1, n2 = l2 ? new_port(VAR, g2) : c2;
          nstore(d, p.nbase, new_pair(n1, n2));
          p.lx1 = l1 ? n1 : n2; p.ly1 = l1 ? c1 : c2;
          p.lx2 = n2; p.ly2 = c2;
          p.nlinks = 1 + (l1 ? 1 : 0) + (l2 ? 1 : 0);
          made = true;
        }
      } else if (rule == GLOB_RULE) {
        // Turn's end: each local end of the redex is wired to a fresh global
        // var, and the redex, now global, goes to the ring.
        const bool la = is_local(p.a), lb = is_local(p.b);
        const uint32_t ga = la ? alloc_run<true>(d, t, t.va, 1) : 1;
        const uint32_t gb = lb ? alloc_run<true>(d, t, t.va, 1) : 1;
        if (!ga || !gb) {
          rc = IR_FATAL;
        } else {
          const Port a2 = la ? new_port(VAR, ga) : p.a, b2 = lb ? new_port(VAR, gb) : p.b;
          ring_put(d, t, new_pair(a2, b2));
          p.lx1 = la ? a2 : b2; p.ly1 = la ? p.a : p.b;
          p.lx2 = b2; p.ly2 = p.b;
          p.nlinks = (la ? 1 : 0) + (lb ? 1 : 0);
          made = true;
        }
      }
    }
    if (!LOCAL || (rule != LEAK_RULE && rule != GLOB_RULE)) switch (rule) {
      case LINK: p.nlinks = 1; break;
      case VOID: p.nlinks = 0; break;
      case ERAS: case ANNI: p.nlinks = 2; break;
      case COMM: {
        // Vars first (taken as NONE), then the nodes, filled right below (no
        // mark); in the block's local net when the lane's slice has room.
        if constexpr (LOCAL) {
          p.vbase = lalloc<true>(t, 4);
          p.nbase = p.vbase ? lalloc<false>(t, 4) : 0;
          if (p.vbase && !p.nbase)
            for (uint32_t i = 0; i < 4; i++) v_store<LOCAL>(d, t, p.vbase + i, 0);
          if (!p.nbase) {
            p.vbase = alloc_run<true>(d, t, t.va, 4);
            p.nbase = p.vbase ? alloc_run<false, false>(d, t, t.na, 4) : 0;
          }
        } else {
          p.vbase = alloc_run<true>(d, t, t.va, 4);
          p.nbase = p.vbase ? alloc_run<false, false>(d, t, t.na, 4) : 0;
        }
        if (!p.vbase || !p.nbase) { rc = IR_FATAL; break; }
        const uint32_t v = p.vbase;
        n_store<LOCAL>(d, t, p.nbase + 0, new_pair(new_port(VAR, v + 0), new_port(VAR, v + 1)));
        n_store<LOCAL>(d, t, p.nbase + 1, new_pair(new_port(VAR, v + 2), new_port(VAR, v + 3)));
        n_store<LOCAL>(d, t, p.nbase + 2, new_pair(new_port(VAR, v + 0), new_port(VAR, v + 2)));
        n_store<LOCAL>(d, t, p.nbase + 3, new_pair(new_port(VAR, v + 1), new_port(VAR, v + 3)));
        made = true;
        p.nlinks = 4;
        break;
      }
      case OPER: {
        Port b1 = get_fst(p.B);
        p.oper_num = get_tag(b1) == NUM;
        p.nlinks = 1;
        if (p.oper_num) {
          p.cv = operate(get_val(p.a), get_val(b1));
        } else {
          if constexpr (LOCAL) {
            p.nbase = lalloc<false>(t, 1);
            if (!p.nbase) p.nbase = alloc_run<false, false>(d, t, t.na, 1);
          } else {
            p.nbase = alloc_run<false, false>(d, t, t.na, 1);
          }
          if (!p.nbase) { rc = IR_FATAL; break; }
          Port b2 = get_snd(p.B);
          if constexpr (LOCAL) if (p.nbase >= LOCAL_WORDS && is_local(b2)) {
            // Local-net variant: a fresh global node cannot hold a local
            // port; a fresh global var takes its place, wired to it by one
            // more link.
            const uint32_t g = alloc_run<true>(d, t, t.va, 1);
            if (!g) { rc = IR_FATAL; break; }
            p.lx1 = new_port(VAR, g); p.ly1 = b2; p.nlinks = 2;
            b2 = p.lx1;
          }
          n_store<LOCAL>(d, t, p.nbase, new_pair(p.a, b2));
          made = true;
        }
        break;
      }
      case SWIT: {
        uint32_t n = get_u24(get_val(p.a));
        p.nlinks = 1;
        if constexpr (LOCAL) {
          p.nbase = lalloc<false>(t, n == 0 ? 1 : 2);
          if (!p.nbase) p.nbase = alloc_run<false, false>(d, t, t.na, n == 0 ? 1 : 2);
        } else {
          p.nbase = alloc_run<false, false>(d, t, t.na, n == 0 ? 1 : 2);
        }
        if (!p.nbase) { rc = IR_FATAL; break; }
        Port b2 = get_snd(p.B);
        if constexpr (LOCAL) if (p.nbase >= LOCAL_WORDS && is_local(b2)) {  // as in OPER
          const uint32_t g = alloc_run<true>(d, t, t.va, 1);
          if (!g) { rc = IR_FATAL; break; }
          p.lx1 = new_port(VAR, g); p.ly1 = b2; p.nlinks = 2;
          b2 = p.lx1;
        }
        if (n == 0) {
          n_store<LOCAL>(d, t, p.nbase, new_pair(b2, new_port(ERA, 0)));
        } else {
          n_store<LOCAL>(d, t, p.nbase, new_pair(new_port(ERA, 0), new_port(CON, p.nbase + 1)));
          n_store<LOCAL>(d, t, p.nbase + 1, new_pair(new_port(NUM, new_u24(n - 1)), b2));
        }
        made = true;
        break;
      }
      default: {  // CALL (src/hvm.c:865-898)
        p.contig = p.node_len <= CHUNK && p.vars_len <= CHUNK;
        bool loc = false;
        if (LOCAL && p.node_len <= LOCAL_SLICE && p.vars_len <= LOCAL_SLICE) {
          // The def's words in the lane's slice of the local net, if it has room.
          p.vbase = p.vars_len ? lalloc<true>(t, p.vars_len) : 0;
          p.nbase = (p.node_len && (p.vbase || !p.vars_len)) ? lalloc<false>(t, p.node_len) : 0;
          loc = (!p.vars_len || p.vbase) && (!p.node_len || p.nbase);
          if (!loc && p.vbase)
            for (uint32_t i = 0; i < p.vars_len; i++) v_store<LOCAL>(d, t, p.vbase + i, 0);
          if (loc) p.contig = true;
        }
        if (p.contig && !loc) {
          // Vars first (taken as NONE), then the nodes: one contiguous run
          // each, so relocation is base + index. In a fragmented space the
          // runs may not be found quickly; then the words are taken one by
          // one and relocated through the per-thread tables.
          const uint32_t soft = d.tables ? SOFT_RUN_CHUNKS : 0;
          p.vbase = p.vars_len ? alloc_run<true>(d, t, t.va, p.vars_len, soft) : 0;
          // The node run is the interaction's last node allocation and is
          // filled right below, so its words need no mark.
          p.nbase = (p.node_len && (p.vbase || !p.vars_len)) ? alloc_run<false, false>(d, t, t.na, p.node_len, soft) : 0;
          if ((p.vars_len && !p.vbase) || (p.node_len && !p.nbase)) {
            if (!d.tables) { rc = IR_FATAL; break; }
            if (p.vbase) {  // give back
              for (uint32_t i = 0; i < p.vars_len; i++) vstore(d, p.vbase + i, 0);
              t.live_vars -= p.vars_len;
            }
            p.contig = false;
          }
        }
        if (!p.contig) {
          for (uint32_t i = 0; i < p.node_len && rc == IR_DONE; i++) {
            uint32_t at = alloc_node(d, t);
            if (!at) rc = IR_FATAL;
            d.nloc[(size_t)i * d.nthreads + t.gid] = at;
          }
          for (uint32_t i = 0; i < p.vars_len && rc == IR_DONE; i++) {
            uint32_t at = alloc_var(d, t);
            if (!at) rc = IR_FATAL;
            d.vloc[(size_t)i * d.nthreads + t.gid] = at;
          }
          if (rc != IR_DONE) break;
        }
        const Pair* nodes = d.book + p.off + p.rbag_len;
        // A fast path leaves out the nodes it consumes: the root (ANNI), or
        // the root, the switch and its CON (SWITCH).
        const uint32_t skip = !FAST || !p.fast ? 0u
                            : p.fast == 1 ? 1u << fast_field(p.fpad, 0)
                            : (1u << fast_field(p.fpad, 0)) | (1u << fast_field(p.fpad, 1)) | (1u << fast_field(p.fpad, 2));
#ifdef HVM_COMPILED_CALLS
        if (!(d.compiled && p.contig && compiled_call_nodes(d, p.fid, p.nbase, p.vbase)))
#endif
        for (uint32_t i = 0; i < p.node_len; i++) {
          uint32_t at = p.contig ? p.nbase + i : d.nloc[(size_t)i * d.nthreads + t.gid];
          if ((skip >> i) & 1u) {
            if (!p.contig) nstore(d, at, 0);  // taken (marked) one by one: give it back
            continue;
          }
          Pair q = book_pair(&nodes[i]);
          n_store<LOCAL>(d, t, at, new_pair(relocate(d, t.gid, p, get_fst(q)), relocate(d, t.gid, p, get_snd(q))));
        }
        t.live_nodes -= __popc(skip);
        if (FAST && p.fast) {
          // The caller's node: consumed, or reused as (#(X-1) R).
          if (p.fast == 3) {
            nstore(d, get_val(p.b), new_pair(new_port(NUM, new_u24(get_u24(get_val(get_fst(p.B))) - 1)), get_snd(p.B)));
          } else {
            nstore(d, get_val(p.b), 0);
            t.live_nodes--;
          }
          if (p.fast >= 2) {  // the switch's result var r is consumed with it
            const uint32_t r = fast_field(p.fpad, 3);
            vstore(d, p.contig ? p.vbase + r : d.vloc[(size_t)r * d.nthreads + t.gid], 0);
            t.live_vars--;
          }
        }
        made = p.node_len > 0 || p.vars_len > 0;
        p.nlinks = p.rbag_len + (p.joined ? 0 : 1) + (FAST && p.fast ? 1 : 0);
        break;
      }
    }
    if (rc == IR_FATAL) {
      set_status(d, ST_OOM_NODES, t.gid);  // a node or var page list / pool ran out
      t.dead = true;
    }
  }

  long long c2 = 0, c3 = 0;
  if (wp) { __syncwarp(); c2 = clock64(); }
  // 5. Fresh words only need to be visible to other threads before the first
  //    exchange that could publish them; pairs wired without an exchange
  //    (redexes pushed to the lane's own deque) need no fence. So the fence
  //    is taken once, lazily, before the first exchange step below.
  if (made) t.dirty = true;
  bool fence_due = __any_sync(0xFFFFFFFFu, t.dirty);
  if (wp) c3 = clock64();
  uint32_t steps = 0;

  // 6. link: two independent link chains per lane, one exchange each per
  //    step, so a rule's pairs are wired two at a time.
  if (rc != IR_DONE) p.nlinks = 0;
  uint32_t next = 0;
  Slot s0, s1;
  s0.busy = s1.busy = false;
  for (uint32_t guard = 0; guard < (1u << 24); guard++) {
    slot_fill<FAST, LOCAL>(d, t, p, next, s0);
    slot_fill<FAST, LOCAL>(d, t, p, next, s1);
    if (!__any_sync(0xFFFFFFFFu, s0.busy || s1.busy)) break;
    if (fence_due) { __threadfence(); fence_due = false; t.dirty = false; }
    steps++;
    slot_leak<LOCAL>(d, t, s0);
    slot_leak<LOCAL>(d, t, s1);
    uint32_t a0, a1;
    Port q0, q1;
    slot_request(s0, a0, q0);
    slot_request(s1, a1, q1);
    Port g0 = s0.busy ? v_exch<LOCAL>(d, t, a0, q0) : 0;
    Port g1 = s1.busy ? v_exch<LOCAL>(d, t, a1, q1) : 0;
    slot_result<LOCAL>(d, t, s0, a0, g0);
    slot_result<LOCAL>(d, t, s1, a1, g1);
  }

  if (wp) {
    long long c4 = clock64();
    wp->v[PROF_ROUNDS] += 1;
    wp->v[PROF_LANES] += __popc(__ballot_sync(0xFFFFFFFFu, has));
    wp->v[PROF_STEPS] += steps;
    wp->v[PROF_CYC_ROUND] += c4 - c0;
    wp->v[PROF_CYC_LOAD] += c1 - c0;
    wp->v[PROF_CYC_WRITE] += c2 - c1;
    wp->v[PROF_CYC_FENCE] += c3 - c2;
    wp->v[PROF_CYC_LINK] += c4 - c3;
  }
  if (has && rc == IR_RETRY) { push<LOCAL>(d, t, r); t.retries++; }
  if (LOCAL && has && rc == IR_DONE && rule == LEAK_RULE) t.hist[LINK]++;  // LEAK copies (not interactions)
  if (has && rc == IR_DONE && p.counted) {
    t.itrs++;
    if (!HREG) {
      t.hist[rule]++;
    } else {
      switch (rule) {
        case CALL: t.hist[CALL]++; break;
        case VOID: t.hist[VOID]++; break;
        case ERAS: t.hist[ERAS]++; break;
        case ANNI: t.hist[ANNI]++; break;
        case COMM: t.hist[COMM]++; break;
        case OPER: t.hist[OPER]++; break;
        default: t.hist[SWIT]++; break;
      }
    }
    if (FAST && p.fast) {  // the interactions a fast path performs in place (src/cmp.rs:147, 191, 220, 253)
      t.itrs += p.fast == 1 ? 1 : 3;
      t.hist[ANNI] += p.fast == 1 ? 1 : 2;
      if (p.fast >= 2) t.hist[SWIT]++;
    }
  }
  return rc;
}

HVM_NS_END
