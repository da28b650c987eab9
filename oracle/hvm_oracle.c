/* hvm_oracle.c — TEST INFRASTRUCTURE ONLY: the CPU oracle for the HVM2
 * evaluator hot path.
 *
 * A plain-C restatement of the reference's CPU runtime, the one `hvm run-c`
 * runs (src/hvm.c + src/run.c). Only the test suite, the smoke check and the
 * CPU-baseline leg of bench.py run it, as the checker; the product never
 * links or calls it. Each function names the reference lines it follows.
 *
 * What it computes, exactly as the reference does:
 *   - the eight interaction rules on packed 32-bit ports / 64-bit node pairs,
 *     with the reference's lock-free linker and availability re-tries;
 *   - per-thread high-priority stacks plus a stealable low-priority bag per
 *     thread (work stealing from the left neighbour), with an idle counter for
 *     termination (src/hvm.c:1127-1185);
 *   - the post-normalisation readback of a lambda-encoded constructor, which
 *     re-normalises every REF it meets and so adds to the interaction count
 *     (src/run.c:67-97, src/hvm.c:1233-1243);
 *   - the printed result and `- ITRS` / `- TIME` / `- MIPS` lines
 *     (src/hvm.c:1535-1699, 1774-1785).
 * IO builtins (src/run.c:123-735) are out of scope: an IO_CALL stops the loop.
 *
 * Parity is pinned by tests against the reference's own C runtime compiled
 * from its sources (oracle/_ref) and against the reference's snapshots.
 *
 * Usage: hvm_oracle [-t threads] [-w] [-n] <book.bin>
 *   -w  count algorithmic bytes (one worker)   -n  print the normalisation time in ns
 */
#include <inttypes.h>
#include <math.h>
#include <pthread.h>
#include <sched.h>
#include <stdatomic.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef uint8_t u8;
typedef uint32_t u32;
typedef uint64_t u64;
typedef int32_t i32;
typedef u32 Port;
typedef u64 Pair;
typedef u32 Numb;

enum { VAR, REF, ERA, NUM, CON, DUP, OPR, SWI };
enum { LINK, CALL, VOID, ERAS, ANNI, COMM, OPER, SWIT };
enum {
  TY_SYM, TY_U24, TY_I24, TY_F24, OP_ADD, OP_SUB, FP_SUB, OP_MUL, OP_DIV, FP_DIV, OP_REM,
  FP_REM, OP_EQ, OP_NEQ, OP_LT, OP_GT, OP_AND, OP_OR, OP_XOR, OP_SHL, FP_SHL, OP_SHR, FP_SHR
};

#define ROOT 0xFFFFFFF8u
#define NONE 0xFFFFFFFFu

/* Capacities of src/hvm.c:119-125 / 135-136. */
#define HI_CAP (1ul << 16)
#define LO_CAP (1ul << 24)
#define NODE_SPACE (1ul << 29)
#define VARS_SPACE (1ul << 29)
#define DEF_MAX 0xFFF
#define NUM_DEFS 0x4000

/* ---- encodings (src/hvm.c:197-348) ---- */
static inline Port mk_port(u32 tag, u32 val) { return (val << 3) | tag; }
static inline u32 tag_of(Port p) { return p & 7; }
static inline u32 val_of(Port p) { return p >> 3; }
static inline Pair mk_pair(Port a, Port b) { return ((u64)b << 32) | a; }
static inline Port fst_of(Pair p) { return (Port)p; }
static inline Port snd_of(Pair p) { return (Port)(p >> 32); }

static const u8 RULES[8][8] = {
  {LINK, LINK, LINK, LINK, LINK, LINK, LINK, LINK},
  {LINK, VOID, VOID, VOID, CALL, CALL, CALL, CALL},
  {LINK, VOID, VOID, VOID, ERAS, ERAS, ERAS, ERAS},
  {LINK, VOID, VOID, VOID, ERAS, ERAS, OPER, SWIT},
  {LINK, CALL, ERAS, ERAS, ANNI, COMM, COMM, COMM},
  {LINK, CALL, ERAS, ERAS, COMM, ANNI, COMM, COMM},
  {LINK, CALL, ERAS, OPER, COMM, COMM, ANNI, COMM},
  {LINK, CALL, ERAS, SWIT, COMM, COMM, COMM, ANNI},
};
static inline u32 rule_of(Port a, Port b) { return RULES[tag_of(a)][tag_of(b)]; }
static inline bool shrinking(u32 rule) { return (0x1Du >> rule) & 1u; }

/* ---- numbers (src/hvm.c:354-558) ---- */
static inline u32 f2u(float f) { u32 u; memcpy(&u, &f, 4); return u; }
static inline float u2f(u32 u) { float f; memcpy(&f, &u, 4); return f; }
static inline Numb n_sym(u32 v) { return (v << 5) | TY_SYM; }
static inline u32 n_symv(Numb w) { return w >> 5; }
static inline Numb n_u24(u32 v) { return (v << 5) | TY_U24; }
static inline u32 n_u24v(Numb w) { return w >> 5; }
static inline Numb n_i24(i32 v) { return ((u32)v << 5) | TY_I24; }
static inline i32 n_i24v(Numb w) { return ((i32)(w << 3)) >> 8; }
static inline u32 n_typ(Numb w) { return w & 0x1F; }
static Numb n_f24(float x) {
  u32 bits = f2u(x), hi = bits >> 8, lo = bits & 0xFF, nan = isnan(x) ? 1u : 0u;
  hi += (!nan) & ((lo - ((lo >> 7) & (hi == 0))) >> 7);
  hi |= nan;
  return (hi << 5) | TY_F24;
}
static inline float n_f24v(Numb w) { return u2f((w << 3) & 0xFFFFFF00u); }
static inline bool n_isnum(Numb w) { return n_typ(w) >= TY_U24 && n_typ(w) <= TY_F24; }
static inline bool n_iscast(Numb w) { return n_typ(w) == TY_SYM && n_symv(w) >= TY_U24 && n_symv(w) <= TY_F24; }
static inline float clampf(float x, float lo, float hi) { float t = x < lo ? lo : x; return t > hi ? hi : t; }

static Numb n_cast(Numb a, Numb b) {
  u32 to = n_symv(a), from = n_typ(b);
  const float umax = (float)(1 << 24) - 1, imax = (float)(1 << 23) - 1, imin = (float)(i32)((~0u) << 23);
  if (to == TY_U24) {
    if (from == TY_U24) return b;
    if (from == TY_I24) return n_u24((u32)n_i24v(b));
    if (from == TY_F24) { float v = n_f24v(b); return isnan(v) ? n_u24(0) : n_u24((u32)clampf(v, 0.0f, umax)); }
  }
  if (to == TY_I24) {
    if (from == TY_U24) return n_i24((i32)n_u24v(b));
    if (from == TY_I24) return b;
    if (from == TY_F24) { float v = n_f24v(b); return isnan(v) ? n_i24(0) : n_i24((i32)clampf(v, imin, imax)); }
  }
  if (to == TY_F24) {
    if (from == TY_U24) return n_f24((float)n_u24v(b));
    if (from == TY_I24) return n_f24((float)n_i24v(b));
    if (from == TY_F24) return b;
  }
  return n_u24(0);
}

static Numb n_operate(Numb a, Numb b) {
  u32 at = n_typ(a), bt = n_typ(b);
  if (at == TY_SYM && bt == TY_SYM) return n_u24(0);
  if (n_iscast(a) && n_isnum(b)) return n_cast(a, b);
  if (n_iscast(b) && n_isnum(a)) return n_cast(b, a);
  if (at == TY_SYM) return (b & ~0x1Fu) | n_symv(a);
  if (bt == TY_SYM) return (a & ~0x1Fu) | n_symv(b);
  if (at >= OP_ADD && bt >= OP_ADD) return n_u24(0);
  if (at < OP_ADD && bt < OP_ADD) return n_u24(0);
  u32 op = at >= OP_ADD ? at : bt, ty = at >= OP_ADD ? bt : at;
  if (at < OP_ADD) { Numb t = a; a = b; b = t; }
  if (ty == TY_U24) {
    u32 x = n_u24v(a), y = n_u24v(b);
    switch (op) {
      case OP_ADD: return n_u24(x + y);   case OP_SUB: return n_u24(x - y);
      case FP_SUB: return n_u24(y - x);   case OP_MUL: return n_u24(x * y);
      case OP_DIV: return n_u24(y ? x / y : 0); case FP_DIV: return n_u24(x ? y / x : 0);
      case OP_REM: return n_u24(y ? x % y : 0); case FP_REM: return n_u24(x ? y % x : 0);
      case OP_EQ: return n_u24(x == y);   case OP_NEQ: return n_u24(x != y);
      case OP_LT: return n_u24(x < y);    case OP_GT: return n_u24(x > y);
      case OP_AND: return n_u24(x & y);   case OP_OR: return n_u24(x | y);
      case OP_XOR: return n_u24(x ^ y);
      case OP_SHL: return n_u24(x << (y & 31)); case FP_SHL: return n_u24(y << (x & 31));
      case OP_SHR: return n_u24(x >> (y & 31)); case FP_SHR: return n_u24(y >> (x & 31));
      default: return n_u24(0);
    }
  }
  if (ty == TY_I24) {
    i32 x = n_i24v(a), y = n_i24v(b);
    switch (op) {
      case OP_ADD: return n_i24((i32)((u32)x + (u32)y)); case OP_SUB: return n_i24((i32)((u32)x - (u32)y));
      case FP_SUB: return n_i24((i32)((u32)y - (u32)x)); case OP_MUL: return n_i24((i32)((u32)x * (u32)y));
      case OP_DIV: return n_i24(y ? x / y : 0); case FP_DIV: return n_i24(x ? y / x : 0);
      case OP_REM: return n_i24(y ? x % y : 0); case FP_REM: return n_i24(x ? y % x : 0);
      case OP_EQ: return n_u24(x == y);   case OP_NEQ: return n_u24(x != y);
      case OP_LT: return n_u24(x < y);    case OP_GT: return n_u24(x > y);
      case OP_AND: return n_i24(x & y);   case OP_OR: return n_i24(x | y);
      case OP_XOR: return n_i24(x ^ y);
      default: return n_i24(0);
    }
  }
  if (ty == TY_F24) {
    float x = n_f24v(a), y = n_f24v(b);
    switch (op) {
      case OP_ADD: return n_f24(x + y);   case OP_SUB: return n_f24(x - y);
      case FP_SUB: return n_f24(y - x);   case OP_MUL: return n_f24(x * y);
      case OP_DIV: return n_f24(x / y);   case FP_DIV: return n_f24(y / x);
      case OP_REM: return n_f24(fmodf(x, y)); case FP_REM: return n_f24(fmodf(y, x));
      case OP_EQ: return n_u24(x == y);   case OP_NEQ: return n_u24(x != y);
      case OP_LT: return n_u24(x < y);    case OP_GT: return n_u24(x > y);
      case OP_AND: return n_f24(atan2f(x, y));
      case OP_OR: return n_f24(logf(y) / logf(x));
      case OP_XOR: return n_f24(powf(x, y));
      case OP_SHL: return n_f24((float)sin(x + y));
      case OP_SHR: return n_f24((float)tan(x + y));
      default: return n_f24(0);
    }
  }
  return n_u24(0);
}

/* ---- book (src/hvm.c:1408-1453) ---- */
typedef struct {
  char name[256];
  bool safe;
  u32 rbag_len, node_len, vars_len;
  Port root;
  Pair* rbag;
  Pair* node;
} Def;

static Def* g_defs;
static u32 g_ndefs;

static bool load_book(const u32* w) {
  g_defs = calloc(NUM_DEFS, sizeof(Def));
  g_ndefs = *w++;
  for (u32 k = 0; k < g_ndefs; k++) {
    u32 fid = *w++;
    if (fid >= NUM_DEFS) { fprintf(stderr, "bad fid %u\n", fid); return false; }
    Def* d = &g_defs[fid];
    memcpy(d->name, w, 256); w += 64;
    d->safe = *w++ != 0;
    d->rbag_len = *w++;
    d->node_len = *w++;
    d->vars_len = *w++;
    if (d->rbag_len > DEF_MAX) { fprintf(stderr, "def '%s' has too many redexes: %u\n", d->name, d->rbag_len); return false; }
    if (d->node_len > DEF_MAX) { fprintf(stderr, "def '%s' has too many nodes: %u\n", d->name, d->node_len); return false; }
    d->root = *w++;
    d->rbag = malloc(8 * (d->rbag_len + 1));
    d->node = malloc(8 * (d->node_len + 1));
    memcpy(d->rbag, w, 8 * d->rbag_len); w += 2 * d->rbag_len;
    memcpy(d->node, w, 8 * d->node_len); w += 2 * d->node_len;
  }
  return true;
}

/* ---- net and workers (src/hvm.c:127-183, 589-778) ---- */
typedef struct {
  _Atomic(u64)* node;
  _Atomic(u32)* vars;
  _Atomic(u64)* bags;   /* one low-priority bag of LO_CAP per worker */
  _Atomic(u64) itrs;
  _Atomic(u32) idle;
} Net;

typedef struct {
  u32 id;
  u32 itrs;
  u32 ncur, vcur;       /* allocation cursors within this worker's slice */
  u32 hlen, llen;       /* stack heights */
  u32 steal_at;
  u32 nloc[DEF_MAX], vloc[DEF_MAX];
  Pair* hstack;         /* HI_CAP high-priority redexes */
} Worker;

static Net* g_net;
static Worker** g_workers;

/* Algorithmic bytes (-w, one worker): the fixed word-touch model of the
 * reference's evaluator used as the roofline numerator -- node take 16 B
 * (8 read + 8 write), node create 8 B, var create 4 B, var exchange 8 B
 * (4 + 4), and 16 B per redex (push 8 + pop 8). Allocation scans,
 * availability checks and the readback are not counted. */
static int g_count_bytes;
static int g_precise;  /* -n: also print the normalisation time in ns */
static u64 g_bytes;
static u64 g_atomics;  /* node takes and var exchanges: the atomic operations of the model */
#define COUNT(n) do { if (g_count_bytes) g_bytes += (n); } while (0)
#define COUNT_ATOMIC() do { if (g_count_bytes) g_atomics++; } while (0)
static u32 g_nthreads;
static u64 g_node_slice, g_vars_slice;

static inline void bag_push(Worker* w, Pair r) {
  COUNT(16);
  if (shrinking(rule_of(fst_of(r), snd_of(r)))) {
    w->hstack[w->hlen++] = r;
  } else {
    atomic_store_explicit(&g_net->bags[(u64)w->id * LO_CAP + (w->llen++)], r, memory_order_relaxed);
  }
}

static inline Pair bag_pop(Worker* w) {
  if (w->hlen > 0) return w->hstack[--w->hlen];
  if (w->llen > 0) return atomic_exchange_explicit(&g_net->bags[(u64)w->id * LO_CAP + (--w->llen)], 0, memory_order_relaxed);
  return 0;
}

/* Scans this worker's slice for free slots (src/hvm.c:713-755). */
static u32 grab_nodes(Worker* w, u32 want) {
  u32 got = 0;
  u64 scans = 0;
  while (got < want) {
    u64 at = (u64)w->id * g_node_slice + (w->ncur % g_node_slice);
    Pair cur = atomic_load_explicit(&g_net->node[at], memory_order_relaxed);
    w->ncur++;
    if (at > 0 && cur == 0) w->nloc[got++] = (u32)at;
    if (++scans >= g_node_slice) { fprintf(stderr, "OOM\n"); exit(3); }
  }
  return got;
}

static u32 grab_vars(Worker* w, u32 want) {
  u32 got = 0;
  u64 scans = 0;
  while (got < want) {
    u64 at = (u64)w->id * g_vars_slice + (w->vcur % g_vars_slice);
    Port cur = atomic_load_explicit(&g_net->vars[at], memory_order_relaxed);
    w->vcur++;
    if (at > 0 && cur == 0) w->vloc[got++] = (u32)at;
    if (++scans >= g_vars_slice) { fprintf(stderr, "OOM\n"); exit(3); }
  }
  return got;
}

static inline Pair node_get(u32 i) { return atomic_load_explicit(&g_net->node[i], memory_order_relaxed); }
static inline void node_put(u32 i, Pair p) { COUNT(8); atomic_store_explicit(&g_net->node[i], p, memory_order_relaxed); }
static inline Pair node_swap(u32 i, Pair p) { COUNT(16); COUNT_ATOMIC(); return atomic_exchange_explicit(&g_net->node[i], p, memory_order_relaxed); }
static inline Port var_get(u32 i) { return atomic_load_explicit(&g_net->vars[i], memory_order_relaxed); }
static inline void var_put(u32 i, Port p) { COUNT(4); atomic_store_explicit(&g_net->vars[i], p, memory_order_relaxed); }
static inline Port var_swap(u32 i, Port p) { COUNT(8); COUNT_ATOMIC(); return atomic_exchange_explicit(&g_net->vars[i], p, memory_order_relaxed); }

/* Maps a def-local port to the freshly allocated slots (src/hvm.c:346-362). */
static inline Port relocate(Worker* w, Port p) {
  u32 t = tag_of(p);
  if (t >= CON) return mk_port(t, w->nloc[val_of(p)]);
  if (t == VAR) return mk_port(t, w->vloc[val_of(p)]);
  return p;
}

/* Read-only chase of a substitution chain (src/hvm.c:781-790). */
static Port chase(Port p) {
  while (tag_of(p) == VAR) {
    Port v = var_get(val_of(p));
    if (v == NONE || v == 0) break;
    p = v;
  }
  return p;
}

/* Owning chase: consumes resolved vars on the way (src/hvm.c:793-808). */
static Port follow(Port p) {
  while (tag_of(p) == VAR) {
    Port v = var_swap(val_of(p), NONE);
    if (v == NONE || v == 0) break;
    var_swap(val_of(p), 0);
    p = v;
  }
  return p;
}

/* Lock-free wiring of A ~ B (src/hvm.c:811-840). */
static void wire(Worker* w, Port a, Port b) {
  for (;;) {
    if (tag_of(a) != VAR && tag_of(b) == VAR) { Port t = a; a = b; b = t; }
    if (tag_of(a) != VAR) { bag_push(w, mk_pair(a, b)); return; }
    b = follow(b);
    Port prev = var_swap(val_of(a), b);
    if (prev == NONE) return;
    var_swap(val_of(a), 0);
    a = prev;
  }
}

static inline bool have_room(Worker* w, u32 redexes) {
  u32 lo_free = (u32)(LO_CAP - w->llen), hi_free = (u32)(HI_CAP - w->hlen);
  return (lo_free < hi_free ? lo_free : hi_free) >= redexes;
}

static bool do_eras(Worker* w, Port a, Port b);

/* src/hvm.c:865-898 */
static bool do_call(Worker* w, Port a, Port b) {
  Def* d = &g_defs[val_of(a) & 0xFFFFFFF];
  if (d->safe && tag_of(b) == DUP) return do_eras(w, a, b);
  bool room = have_room(w, d->rbag_len + 1);
  u32 gn = grab_nodes(w, d->node_len), gv = grab_vars(w, d->vars_len);
  if (!room || gn < d->node_len || gv < d->vars_len) return false;
  for (u32 i = 0; i < d->vars_len; i++) var_put(w->vloc[i], NONE);
  for (u32 i = 0; i < d->node_len; i++) {
    Pair p = d->node[i];
    node_put(w->nloc[i], mk_pair(relocate(w, fst_of(p)), relocate(w, snd_of(p))));
  }
  for (u32 i = 0; i < d->rbag_len; i++) {
    Pair p = d->rbag[i];
    wire(w, relocate(w, fst_of(p)), relocate(w, snd_of(p)));
  }
  wire(w, relocate(w, d->root), b);
  return true;
}

/* src/hvm.c:907-929 */
static bool do_eras(Worker* w, Port a, Port b) {
  if (!have_room(w, 2)) return false;
  if (node_get(val_of(b)) == 0) return false;
  Pair B = node_swap(val_of(b), 0);
  wire(w, a, fst_of(B));
  wire(w, a, snd_of(B));
  return true;
}

/* src/hvm.c:932-957 */
static bool do_anni(Worker* w, Port a, Port b) {
  if (!have_room(w, 2)) return false;
  if (node_get(val_of(a)) == 0 || node_get(val_of(b)) == 0) return false;
  Pair A = node_swap(val_of(a), 0), B = node_swap(val_of(b), 0);
  wire(w, fst_of(A), fst_of(B));
  wire(w, snd_of(A), snd_of(B));
  return true;
}

/* src/hvm.c:960-998 */
static bool do_comm(Worker* w, Port a, Port b) {
  bool room = have_room(w, 4);
  grab_nodes(w, 4);
  grab_vars(w, 4);
  if (!room) return false;
  if (node_get(val_of(a)) == 0 || node_get(val_of(b)) == 0) return false;
  Pair A = node_swap(val_of(a), 0), B = node_swap(val_of(b), 0);
  u32* n = w->nloc;
  u32* v = w->vloc;
  for (int i = 0; i < 4; i++) var_put(v[i], NONE);
  node_put(n[0], mk_pair(mk_port(VAR, v[0]), mk_port(VAR, v[1])));
  node_put(n[1], mk_pair(mk_port(VAR, v[2]), mk_port(VAR, v[3])));
  node_put(n[2], mk_pair(mk_port(VAR, v[0]), mk_port(VAR, v[2])));
  node_put(n[3], mk_pair(mk_port(VAR, v[1]), mk_port(VAR, v[3])));
  wire(w, mk_port(tag_of(b), n[0]), fst_of(A));
  wire(w, mk_port(tag_of(b), n[1]), snd_of(A));
  wire(w, mk_port(tag_of(a), n[2]), fst_of(B));
  wire(w, mk_port(tag_of(a), n[3]), snd_of(B));
  return true;
}

/* src/hvm.c:1001-1029 */
static bool do_oper(Worker* w, Port a, Port b) {
  bool room = have_room(w, 1);
  grab_nodes(w, 1);
  if (!room) return false;
  if (node_get(val_of(b)) == 0) return false;
  Pair B = node_swap(val_of(b), 0);
  Port b1 = fst_of(B), b2 = follow(snd_of(B));
  if (tag_of(b1) == NUM) {
    wire(w, mk_port(NUM, n_operate(val_of(a), val_of(b1))), b2);
  } else {
    node_put(w->nloc[0], mk_pair(a, b2));
    wire(w, b1, mk_port(OPR, w->nloc[0]));
  }
  return true;
}

/* src/hvm.c:1032-1063 */
static bool do_swit(Worker* w, Port a, Port b) {
  bool room = have_room(w, 1);
  grab_nodes(w, 2);
  if (!room) return false;
  if (node_get(val_of(b)) == 0) return false;
  u32 n = n_u24v(val_of(a));
  Pair B = node_swap(val_of(b), 0);
  u32* loc = w->nloc;
  if (n == 0) {
    node_put(loc[0], mk_pair(snd_of(B), mk_port(ERA, 0)));
  } else {
    node_put(loc[0], mk_pair(mk_port(ERA, 0), mk_port(CON, loc[1])));
    node_put(loc[1], mk_pair(mk_port(NUM, n_u24(n - 1)), snd_of(B)));
  }
  wire(w, mk_port(CON, loc[0]), fst_of(B));
  return true;
}

/* One interaction (src/hvm.c:1073-1122). */
static void step(Worker* w) {
  Pair r = bag_pop(w);
  if (r == 0) return;
  Port a = fst_of(r), b = snd_of(r);
  u32 rule = rule_of(a, b);
  if (tag_of(a) == REF && b == ROOT) {
    rule = CALL;
  } else if (tag_of(b) < tag_of(a)) {
    Port t = a; a = b; b = t;
  }
  bool ok;
  switch (rule) {
    case LINK: ok = have_room(w, 1); if (ok) wire(w, a, b); break;
    case CALL: ok = do_call(w, a, b); break;
    case VOID: ok = true; break;
    case ERAS: ok = do_eras(w, a, b); break;
    case ANNI: ok = do_anni(w, a, b); break;
    case COMM: ok = do_comm(w, a, b); break;
    case OPER: ok = do_oper(w, a, b); break;
    default:   ok = do_swit(w, a, b); break;
  }
  if (!ok) bag_push(w, r);
  else if (rule != LINK) w->itrs++;
}

/* Spin barrier shared by the workers (src/hvm.c:273-287). */
static _Atomic(u64) g_arrived, g_generation;
static void barrier(void) {
  u64 gen = atomic_load(&g_generation);
  if (atomic_fetch_add(&g_arrived, 1) == g_nthreads - 1) {
    atomic_store(&g_arrived, 0);
    atomic_store(&g_generation, gen + 1);
  } else {
    while (atomic_load(&g_generation) == gen) sched_yield();
  }
}

/* Worker loop with left-neighbour stealing (src/hvm.c:1127-1185). */
static void* work(void* arg) {
  Worker* w = (Worker*)arg;
  atomic_store(&g_net->idle, g_nthreads - 1);
  barrier();
  u32 tick = 0;
  bool busy = w->id == 0;
  for (;;) {
    tick++;
    if (w->hlen + w->llen > 0) {
      if (!busy) atomic_fetch_sub(&g_net->idle, 1);
      busy = true;
      step(w);
    } else {
      if (busy) atomic_fetch_add(&g_net->idle, 1);
      busy = false;
      u32 victim = (w->id + g_nthreads - 1) % g_nthreads;
      u64 at = (u64)victim * LO_CAP + (w->steal_at++);
      Pair got = atomic_exchange_explicit(&g_net->bags[at], 0, memory_order_relaxed);
      if (got != 0) { bag_push(w, got); continue; }
      w->steal_at = 0;
      sched_yield();
      if (tick % 256 == 0 && atomic_load(&g_net->idle) == g_nthreads) break;
    }
  }
  barrier();
  atomic_fetch_add(&g_net->itrs, w->itrs);
  w->itrs = 0;
  return NULL;
}

/* src/hvm.c:1188-1230 */
static void boot(Pair redex) {
  var_put(val_of(ROOT), NONE);
  atomic_store(&g_net->bags[0], redex);
}

/* The boot redex sits in slot 0 of worker 0's bag with no owner height
 * recorded; a worker picks it up by stealing, as in the reference. */
static void normalize(void) {
  pthread_t th[256];
  for (u32 t = 0; t < g_nthreads; t++) pthread_create(&th[t], NULL, work, g_workers[t]);
  for (u32 t = 0; t < g_nthreads; t++) pthread_join(th[t], NULL);
}

/* src/hvm.c:1233-1243 */
static Port expand(Port p) {
  Port saved = var_get(val_of(ROOT));
  Port got = chase(p);
  while (tag_of(got) == REF) {
    boot(mk_pair(got, ROOT));
    normalize();
    got = chase(var_get(val_of(ROOT)));
  }
  var_put(val_of(ROOT), saved);
  return got;
}

/* Lambda-encoded constructor readback (src/run.c:65-97). */
typedef struct { u32 tag, nargs; Port args[16]; } Ctr;
static Ctr read_ctr(Port p) {
  Ctr c;
  c.tag = (u32)-1;
  c.nargs = 0;
  Port lam = expand(p);
  if (tag_of(lam) != CON) return c;
  Pair lam_n = node_get(val_of(lam));
  Port app = expand(fst_of(lam_n));
  if (tag_of(app) != CON) return c;
  Pair app_n = node_get(val_of(app));
  Port arg = expand(fst_of(app_n));
  if (tag_of(arg) != NUM) return c;
  c.tag = n_u24v(val_of(arg));
  for (;;) {
    app = expand(snd_of(app_n));
    if (tag_of(app) != CON) break;
    app_n = node_get(val_of(app));
    arg = expand(fst_of(app_n));
    /* The reference stores into a 16-slot array without a bound; past 16
     * arguments its behaviour is undefined. Here the walk continues (so the
     * same REFs are expanded) and only the first 16 are kept. */
    if (c.nargs < 16) c.args[c.nargs] = arg;
    c.nargs++;
  }
  return c;
}

/* The IO loop, without the IO builtins (src/run.c:740-810). */
static void run_loop(void) {
  Port port = ROOT;
  for (;;) {
    normalize();
    Ctr c = read_ctr(chase(port));
    if (c.nargs < 1 || tag_of(c.args[0]) != CON) break;
    Pair magic = node_get(val_of(c.args[0]));
    if (val_of(fst_of(magic)) != n_u24(0xD0CA11) || val_of(snd_of(magic)) != n_u24(0xFF1FF1)) break;
    if (c.tag == 1) fprintf(stderr, "IO calls are not supported by the oracle\n");
    break;
  }
}

/* ---- printing (src/hvm.c:1535-1699) ---- */
static void print_numb(Numb w) {
  static const char* syms[] = {
    "[u24]", "[i24]", "[f24]", "[+]", "[-]", "[:-]", "[*]", "[/]", "[:/]", "[%]", "[:%]",
    "[=]", "[!]", "[<]", "[>]", "[&]", "[|]", "[^]", "[<<]", "[:<<]", "[>>]", "[:>>]"};
  static const char* ops[] = {
    "+", "-", ":-", "*", "/", ":/", "%", ":%", "=", "!", "<", ">", "&", "|", "^", "<<", ":<<", ">>", ":>>"};
  u32 t = n_typ(w);
  if (t == TY_SYM) {
    u32 s = n_symv(w);
    printf("%s", (s >= 1 && s <= 22) ? syms[s - 1] : "[?]");
  } else if (t == TY_U24) {
    printf("%u", n_u24v(w));
  } else if (t == TY_I24) {
    printf("%+d", n_i24v(w));
  } else if (t == TY_F24) {
    float f = n_f24v(w);
    if (isinf(f)) printf(signbit(f) ? "-inf" : "+inf");
    else if (isnan(f)) printf("+NaN");
    else printf("%.7e", f);
  } else {
    printf("[%s0x%07X]", (t >= OP_ADD && t <= FP_SHR) ? ops[t - OP_ADD] : "?", n_u24v(w));
  }
}

static void print_tree(Port p) {
  Port stack[4096];
  u32 len = 0;
  stack[len++] = p;
  while (len > 0) {
    Port cur = stack[--len];
    u32 t = tag_of(cur);
    if (t >= CON) {
      static const char* open[] = {"(", "{", "$(", "?("};
      static const char close[] = {')', '}', ')', ')'};
      Pair n = node_get(val_of(cur));
      printf("%s", open[t - CON]);
      stack[len++] = mk_port(ERA, (u32)close[t - CON]);
      stack[len++] = snd_of(n);
      stack[len++] = mk_port(ERA, (u32)' ');
      stack[len++] = fst_of(n);
    } else if (t == ERA) {
      if (val_of(cur) != 0) printf("%c", (char)val_of(cur));
      else printf("*");
    } else if (t == VAR) {
      Port got = var_get(val_of(cur));
      if (got != NONE) stack[len++] = got;
      else printf("x%x", val_of(cur));
    } else if (t == NUM) {
      print_numb(val_of(cur));
    } else {
      printf("@%s", g_defs[val_of(cur) & 0xFFFFFFF].name);
    }
  }
}

static u64 now_ns(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (u64)ts.tv_sec * 1000000000ull + (u64)ts.tv_nsec;
}

int main(int argc, char** argv) {
  u32 threads = 1;
  const char* path = NULL;
  for (int i = 1; i < argc; i++) {
    if (!strcmp(argv[i], "-t") && i + 1 < argc) threads = (u32)atoi(argv[++i]);
    else if (!strcmp(argv[i], "-w")) g_count_bytes = 1;
    else if (!strcmp(argv[i], "-n")) g_precise = 1;
    else path = argv[i];
  }
  if (!path || threads < 1 || threads > 256) { fprintf(stderr, "usage: hvm_oracle [-t threads] [-w] [-n] <book.bin>\n"); return 2; }
  if (g_count_bytes && threads != 1) { fprintf(stderr, "-w counts with one worker only\n"); return 2; }
  FILE* f = fopen(path, "rb");
  if (!f) { perror(path); return 2; }
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  u32* buf = malloc((size_t)sz + 4);
  if (fread(buf, 1, (size_t)sz, f) != (size_t)sz) { fprintf(stderr, "read failed\n"); return 2; }
  fclose(f);
  if (!load_book(buf)) { fprintf(stderr, "failed to load book\n"); return 1; }

  g_nthreads = threads;
  g_node_slice = NODE_SPACE / threads;
  g_vars_slice = VARS_SPACE / threads;
  g_net = calloc(1, sizeof(Net));
  g_net->node = calloc(NODE_SPACE, sizeof(u64));
  g_net->vars = calloc(VARS_SPACE, sizeof(u32));
  g_net->bags = calloc((size_t)threads * LO_CAP, sizeof(u64));
  if (!g_net->node || !g_net->vars || !g_net->bags) { fprintf(stderr, "OOM\n"); return 3; }
  g_workers = calloc(threads, sizeof(Worker*));
  for (u32 t = 0; t < threads; t++) {
    Worker* w = calloc(1, sizeof(Worker));
    w->id = t;
    w->ncur = 1;
    w->vcur = 1;
    w->hstack = malloc(HI_CAP * sizeof(Pair));
    g_workers[t] = w;
  }

  u64 t0 = now_ns();
  boot(mk_pair(mk_port(REF, 0), ROOT));
  run_loop();
  u64 t_norm = now_ns();
  int counted = g_count_bytes;
  g_count_bytes = 0;
  printf("Result: ");
  print_tree(follow(ROOT));
  printf("\n");
  double secs = (double)(now_ns() - t0) / 1e9;
  u64 itrs = atomic_load(&g_net->itrs);
  printf("- ITRS: %" PRIu64 "\n", itrs);
  printf("- TIME: %.2fs\n", secs);
  printf("- MIPS: %.2f\n", (double)itrs / secs / 1000000.0);
  if (g_precise) printf("- NORM_NS: %" PRIu64 "\n", t_norm - t0);
  if (counted) printf("- BYTES: %" PRIu64 "\n- ATOMICS: %" PRIu64 "\n", g_bytes, g_atomics);
  return 0;
}
