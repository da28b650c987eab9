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

namespace hvm {

// Device status codes (0 = running / ok). Written once, first error wins.
enum : uint32_t {
  ST_OK = 0,
  ST_OOM_NODES = 1,     // a thread's node slice has no free word
  ST_OOM_VARS = 2,      // a thread's var slice has no free word
  ST_RING_FULL = 3,     // the global redex ring overflowed
  ST_LINK_UNSET = 4,    // a link met a var word that was never created
  ST_LINK_LIMIT = 5,    // a substitution chain exceeded the iteration bound
  ST_BAD_REF = 6,       // a REF to a definition the book does not have
};

// One book definition on the device. Pairs for a def are stored at
// book[off .. off+rbag_len) (redexes) then book[off+rbag_len ..) (nodes).
struct DefHdr {
  uint32_t node_len, rbag_len, vars_len, safe;
  uint32_t root, off, pad0, pad1;
};

// One record per completed turn, written by the turn's last block.
struct TurnRecord {
  unsigned long long t_ns;          // %globaltimer when the turn closed
  unsigned long long itrs;          // cumulative interactions
  unsigned long long pending;       // redexes in the ring for the next turn
  unsigned int dry, stopped;        // dry threads at close; 1 if ended by the dry rule
  unsigned int budget, per_thread;  // the closed turn's budget and static share
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
  unsigned int policy;              // 0 = fixed policy
  unsigned int pad_c[1];
  unsigned long long hist[8];       // interactions per rule (diagnostic)
  unsigned int npool_next;          // next page id of the node pool
  unsigned int vpool_next;          // next page id of the var pool
  TurnRecord* trace;                // per-turn records (null = off)
  unsigned int trace_cap;
};

constexpr Pair NODE_MARK = ~0ull;

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
  uint32_t* nloc;             // CALL scratch: [max_def_nodes][nthreads]
  uint32_t* vloc;             // CALL scratch: [max_def_vars][nthreads]
  uint32_t nthreads;
  uint32_t ndefs;
  const DefHdr* defs;
  const Pair* book;
  Ctl* ctl;
};

// ---- memory access -----------------------------------------------------------

__device__ __forceinline__ Pair nload(const Dev& d, uint32_t i) {
  return (Pair)__ldcg((const unsigned long long*)&d.node[i]);
}
__device__ __forceinline__ void nstore(const Dev& d, uint32_t i, Pair p) {
  __stcg((unsigned long long*)&d.node[i], (unsigned long long)p);
}
__device__ __forceinline__ Port vload(const Dev& d, uint32_t i) { return __ldcg(&d.vars[i & d.vars_mask]); }
__device__ __forceinline__ void vstore(const Dev& d, uint32_t i, Port p) { __stcg(&d.vars[i & d.vars_mask], p); }
__device__ __forceinline__ Port vexch(const Dev& d, uint32_t i, Port p) { return atomicExch(&d.vars[i & d.vars_mask], p); }

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
};

// ---- per-thread state ----------------------------------------------------------

struct TState {
  Pair* stk;                  // this thread's deque in shared memory (stride = blockDim.x)
  uint32_t stride;
  uint32_t lo, len, cap;      // entries lo .. lo+len-1 (mod cap); cap is a power of two
  uint32_t gid;
  Alloc na, va;               // node / var allocators
  unsigned long long base;    // ring index of this turn's first input (overflow check)
  unsigned long long itrs, leak, retries;
  unsigned long long hist[8];
  bool dead;                  // set after a fatal status: stop interacting
};

// Local redex deque: the thread pops and pushes at the top (LIFO, depth
// first, like the reference's per-thread bags); when it is full, the oldest
// half moves to the global ring with one atomic (those are the redexes other
// threads will take first next turn).
__device__ __forceinline__ Pair& slot(TState& t, uint32_t i) {
  return t.stk[(size_t)((t.lo + i) & (t.cap - 1)) * t.stride];
}

__device__ __forceinline__ void spill_oldest(const Dev& d, TState& t, uint32_t k) {
  unsigned long long at = atomicAdd(&d.ctl->tail, (unsigned long long)k);
  if (at + k - t.base > d.ring_mask + 1) { set_status(d, ST_RING_FULL, 0); t.dead = true; return; }
  for (uint32_t i = 0; i < k; i++) d.ring[(at + i) & d.ring_mask] = slot(t, i);
  t.lo = (t.lo + k) & (t.cap - 1);
  t.len -= k;
  t.leak += k;
}

__device__ __forceinline__ void push(const Dev& d, TState& t, Pair r) {
  if (t.len == t.cap) {
    spill_oldest(d, t, t.cap / 2);
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

template <bool VARS>
__device__ __forceinline__ uint32_t chunk_mask(const Dev& d, uint32_t base) {
  uint32_t m = 0;
  if (!VARS) {
    const ulonglong2* p = (const ulonglong2*)&d.node[base];
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      ulonglong2 v = __ldcg(p + k);
      m |= (v.x == 0 ? 1u : 0u) << (2 * k);
      m |= (v.y == 0 ? 1u : 0u) << (2 * k + 1);
    }
    if (base == 0) m &= ~1u;
    if (base + 8 > d.node_mask) m &= ~(1u << (d.node_mask - base));  // never the MARK word
  } else {
    const uint4* p = (const uint4*)&d.vars[base];
    #pragma unroll
    for (int k = 0; k < 4; k++) {
      uint4 v = __ldcg(p + k);
      m |= (v.x == 0 ? 1u : 0u) << (4 * k);
      m |= (v.y == 0 ? 1u : 0u) << (4 * k + 1);
      m |= (v.z == 0 ? 1u : 0u) << (4 * k + 2);
      m |= (v.w == 0 ? 1u : 0u) << (4 * k + 3);
    }
    if (base == 0) m &= ~1u;
    if (base + 16 > d.vars_mask) m &= ~(1u << (d.vars_mask - base));  // ROOT
  }
  return m;
}

template <bool VARS>
__device__ __forceinline__ uint32_t alloc_word(const Dev& d, TState& t, Alloc& a) {
  const PagedSpace& sp = VARS ? d.vspace : d.nspace;
  const uint32_t chunk_words = VARS ? 16u : 8u;
  const uint32_t page_words = 1u << sp.page_log2;
  const uint32_t chunks_per_page = page_words / chunk_words;
  for (uint32_t guard = 0; guard < (1u << 22); guard++) {
    if (a.mask) {
      uint32_t b = __ffs(a.mask) - 1;
      a.mask &= a.mask - 1;
      uint32_t at = a.chunk + b;
      if (VARS) vstore(d, at, NONE); else nstore(d, at, NODE_MARK);
      return at;
    }
    // Next chunk: within the page, then the next owned page, then a new page.
    if (a.off >= page_words) {
      a.off = 0;
      if (a.dry_chunks >= 2 * chunks_per_page || a.count == 1 && a.dry_chunks >= chunks_per_page) {
        if (a.count >= sp.max_pages) return 0;
        uint32_t fresh = atomicAdd(pool_counter(d, VARS), 1u);
        if (fresh >= (VARS ? d.vpool_end : d.npool_end)) return 0;
        sp.lists[(size_t)t.gid * sp.max_pages + a.count] = fresh;
        a.pos = a.count;
        a.count++;
        sp.counts[t.gid] = a.count;
        a.page = fresh;
        a.dry_chunks = 0;
      } else {
        a.pos = a.pos + 1 == a.count ? 0 : a.pos + 1;
        a.page = __ldcg(&sp.lists[(size_t)t.gid * sp.max_pages + a.pos]);
      }
    }
    a.chunk = (a.page << sp.page_log2) + a.off;
    a.off += chunk_words;
    a.mask = chunk_mask<VARS>(d, a.chunk);
    a.dry_chunks = a.mask ? 0 : a.dry_chunks + 1;
  }
  return 0;
}

__device__ __forceinline__ uint32_t alloc_node(const Dev& d, TState& t) { return alloc_word<false>(d, t, t.na); }
__device__ __forceinline__ uint32_t alloc_var(const Dev& d, TState& t) { return alloc_word<true>(d, t, t.va); }

// Loads a thread's allocator state at turn start; it resumes at the chunk it
// was scanning when the previous turn ended.
template <bool VARS>
__device__ __forceinline__ void alloc_load(const PagedSpace& sp, uint32_t gid, Alloc& a) {
  const uint32_t chunk_words = VARS ? 16u : 8u;
  a.pos = sp.pos[gid];
  a.off = sp.off[gid];
  a.count = sp.counts[gid];
  a.page = sp.lists[(size_t)gid * sp.max_pages + a.pos];
  a.off = a.off >= chunk_words ? a.off - chunk_words : 0;
  a.chunk = 0;
  a.mask = 0;
  a.dry_chunks = 0;
}

__device__ __forceinline__ void alloc_save(const PagedSpace& sp, uint32_t gid, const Alloc& a) {
  sp.pos[gid] = a.pos;
  sp.off[gid] = a.off;
}

// ---- linking (src/hvm.c:784-840) ----------------------------------------------

// Follows a var chain, consuming every resolved var on the way.
__device__ __forceinline__ Port enter(const Dev& d, Port p) {
  for (uint32_t guard = 0; guard < (1u << 24) && get_tag(p) == VAR; guard++) {
    Port v = vexch(d, get_val(p), NONE);
    if (v == NONE || v == 0) break;
    vstore(d, get_val(p), 0);
    p = v;
  }
  return p;
}

// Atomically wires A ~ B: publishes a substitution, or makes a redex when
// both sides are non-vars.
__device__ void link(const Dev& d, TState& t, Port A, Port B) {
  for (uint32_t guard = 0; guard < (1u << 24); guard++) {
    if (get_tag(A) != VAR && get_tag(B) == VAR) { Port x = A; A = B; B = x; }
    if (get_tag(A) != VAR) { push(d, t, new_pair(A, B)); return; }
    B = enter(d, B);
    Port prev = vexch(d, get_val(A), B);
    if (prev == NONE) return;
    if (prev == 0) { set_status(d, ST_LINK_UNSET, get_val(A)); t.dead = true; return; }
    vstore(d, get_val(A), 0);
    A = prev;
  }
  set_status(d, ST_LINK_LIMIT, 0);
  t.dead = true;
}

// ---- interactions (src/hvm.c:852-1122) -----------------------------------------

enum : int { IR_DONE = 0, IR_RETRY = 1, IR_FATAL = 2 };

// Publishes this thread's node/var creations before they become reachable
// from another thread through a link.
__device__ __forceinline__ void publish() { __threadfence(); }

__device__ __forceinline__ int rule_eras(const Dev& d, TState& t, Port a, Port b) {
  Pair B = nload(d, get_val(b));
  if (B == 0) return IR_RETRY;
  nstore(d, get_val(b), 0);
  link(d, t, a, get_fst(B));
  link(d, t, a, get_snd(B));
  return IR_DONE;
}

__device__ __forceinline__ int rule_anni(const Dev& d, TState& t, Port a, Port b) {
  Pair A = nload(d, get_val(a));
  Pair B = nload(d, get_val(b));
  if (A == 0 || B == 0) return IR_RETRY;
  nstore(d, get_val(a), 0);
  nstore(d, get_val(b), 0);
  link(d, t, get_fst(A), get_fst(B));
  link(d, t, get_snd(A), get_snd(B));
  return IR_DONE;
}

__device__ __forceinline__ int rule_comm(const Dev& d, TState& t, Port a, Port b) {
  Pair A = nload(d, get_val(a));
  Pair B = nload(d, get_val(b));
  if (A == 0 || B == 0) return IR_RETRY;
  uint32_t n0 = alloc_node(d, t), n1 = alloc_node(d, t), n2 = alloc_node(d, t), n3 = alloc_node(d, t);
  if (!n0 || !n1 || !n2 || !n3) { set_status(d, ST_OOM_NODES, t.gid); return IR_FATAL; }
  uint32_t v0 = alloc_var(d, t), v1 = alloc_var(d, t), v2 = alloc_var(d, t), v3 = alloc_var(d, t);
  if (!v0 || !v1 || !v2 || !v3) { set_status(d, ST_OOM_VARS, t.gid); return IR_FATAL; }
  nstore(d, get_val(a), 0);
  nstore(d, get_val(b), 0);
  nstore(d, n0, new_pair(new_port(VAR, v0), new_port(VAR, v1)));
  nstore(d, n1, new_pair(new_port(VAR, v2), new_port(VAR, v3)));
  nstore(d, n2, new_pair(new_port(VAR, v0), new_port(VAR, v2)));
  nstore(d, n3, new_pair(new_port(VAR, v1), new_port(VAR, v3)));
  publish();
  link(d, t, new_port(get_tag(b), n0), get_fst(A));
  link(d, t, new_port(get_tag(b), n1), get_snd(A));
  link(d, t, new_port(get_tag(a), n2), get_fst(B));
  link(d, t, new_port(get_tag(a), n3), get_snd(B));
  return IR_DONE;
}

__device__ __forceinline__ int rule_oper(const Dev& d, TState& t, Port a, Port b) {
  Pair B = nload(d, get_val(b));
  if (B == 0) return IR_RETRY;
  nstore(d, get_val(b), 0);
  Port b1 = get_fst(B);
  Port b2 = enter(d, get_snd(B));
  if (get_tag(b1) == NUM) {
    link(d, t, new_port(NUM, operate(get_val(a), get_val(b1))), b2);
  } else {
    uint32_t n0 = alloc_node(d, t);
    if (!n0) { set_status(d, ST_OOM_NODES, t.gid); return IR_FATAL; }
    nstore(d, n0, new_pair(a, b2));
    publish();
    link(d, t, b1, new_port(OPR, n0));
  }
  return IR_DONE;
}

__device__ __forceinline__ int rule_swit(const Dev& d, TState& t, Port a, Port b) {
  Pair B = nload(d, get_val(b));
  if (B == 0) return IR_RETRY;
  uint32_t n = get_u24(get_val(a));
  uint32_t n0 = alloc_node(d, t);
  uint32_t n1 = n == 0 ? 1u : alloc_node(d, t);
  if (!n0 || !n1) { set_status(d, ST_OOM_NODES, t.gid); return IR_FATAL; }
  nstore(d, get_val(b), 0);
  if (n == 0) {
    nstore(d, n0, new_pair(get_snd(B), new_port(ERA, 0)));
  } else {
    nstore(d, n0, new_pair(new_port(ERA, 0), new_port(CON, n1)));
    nstore(d, n1, new_pair(new_port(NUM, new_u24(n - 1)), get_snd(B)));
  }
  publish();
  link(d, t, new_port(CON, n0), get_fst(B));
  return IR_DONE;
}

__device__ __forceinline__ Port relocate(const Dev& d, const TState& t, Port p) {
  Tag tag = get_tag(p);
  if (tag >= CON) return new_port(tag, d.nloc[(size_t)get_val(p) * d.nthreads + t.gid]);
  if (tag == VAR) return new_port(VAR, d.vloc[(size_t)get_val(p) * d.nthreads + t.gid]);
  return p;
}

__device__ int rule_call(const Dev& d, TState& t, Port a, Port b) {
  uint32_t fid = get_val(a) & 0xFFFFFFFu;
  if (fid >= d.ndefs) { set_status(d, ST_BAD_REF, fid); return IR_FATAL; }
  const DefHdr h = d.defs[fid];
  // Copy optimisation: a safe REF meeting a DUP is duplicated like an eraser.
  if (h.safe && get_tag(b) == DUP) return rule_eras(d, t, a, b);
  for (uint32_t i = 0; i < h.node_len; i++) {
    uint32_t at = alloc_node(d, t);
    if (!at) { set_status(d, ST_OOM_NODES, t.gid); return IR_FATAL; }
    d.nloc[(size_t)i * d.nthreads + t.gid] = at;
  }
  for (uint32_t i = 0; i < h.vars_len; i++) {
    uint32_t at = alloc_var(d, t);  // claimed as NONE: created
    if (!at) { set_status(d, ST_OOM_VARS, t.gid); return IR_FATAL; }
    d.vloc[(size_t)i * d.nthreads + t.gid] = at;
  }
  const Pair* nodes = d.book + h.off + h.rbag_len;
  for (uint32_t i = 0; i < h.node_len; i++) {
    Pair p = __ldg((const unsigned long long*)&nodes[i]);
    nstore(d, d.nloc[(size_t)i * d.nthreads + t.gid],
           new_pair(relocate(d, t, get_fst(p)), relocate(d, t, get_snd(p))));
  }
  publish();
  const Pair* rbag = d.book + h.off;
  for (uint32_t i = 0; i < h.rbag_len; i++) {
    Pair p = __ldg((const unsigned long long*)&rbag[i]);
    link(d, t, relocate(d, t, get_fst(p)), relocate(d, t, get_snd(p)));
  }
  link(d, t, relocate(d, t, h.root), b);
  return IR_DONE;
}

// One interaction on redex `r` (src/hvm.c:1073-1122). Returns the rule run,
// or -1 when the redex was pushed back for a re-try.
__device__ __forceinline__ int interact(const Dev& d, TState& t, Pair r) {
  Port a = get_fst(r), b = get_snd(r);
  Rule rule = get_rule(a, b);
  if (get_tag(a) == REF && b == ROOT) {
    rule = CALL;
  } else if (should_swap(a, b)) {
    Port x = a; a = b; b = x;
  }
  int rc;
  switch (rule) {
    case LINK: link(d, t, a, b); rc = IR_DONE; break;
    case CALL: rc = rule_call(d, t, a, b); break;
    case VOID: rc = IR_DONE; break;
    case ERAS: rc = rule_eras(d, t, a, b); break;
    case ANNI: rc = rule_anni(d, t, a, b); break;
    case COMM: rc = rule_comm(d, t, a, b); break;
    case OPER: rc = rule_oper(d, t, a, b); break;
    default:   rc = rule_swit(d, t, a, b); break;
  }
  if (rc == IR_RETRY) {
    push(d, t, r);
    t.retries++;
    return -1;
  }
  if (rc == IR_FATAL) { t.dead = true; return -1; }
  if (rule != LINK) { t.itrs++; t.hist[rule]++; }
  return rule;
}

}  // namespace hvm
