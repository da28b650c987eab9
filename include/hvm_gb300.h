/* hvm_gb300.h — C ABI of the GB300-native HVM2 evaluator (libhvm_gb300.so).
 *
 * Plain C types only: pointers, sizes and fixed-width integers. Every entry
 * point names the reference interface it replaces or extends.
 */
#ifndef HVM_GB300_H
#define HVM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Drop-in entry point ---------------------------------------------------
 *
 * Replaces the reference's CUDA runtime entry point
 *   `extern "C" void hvm_cu(u32* book_buffer)`      (src/hvm.cu:2320)
 * bound from Rust as
 *   `extern "C" { fn hvm_cu(book_buffer: *const u32); }`  (src/main.rs:17-20)
 * `book_buffer` is the serialized Book (src/hvm.rs:957-1003). The call loads
 * the book, normalises `@main`, and prints on stdout, as the reference does:
 *   Result: <tree>
 *   - ITRS: <interactions>
 *   - LEAK: <redexes moved between threads through the global ring>
 *   - TIME: <seconds>s
 *   - MIPS: <million interactions per second>
 * A book the loader rejects prints "failed to load book" on stderr and
 * returns (src/hvm.cu:2325-2328); a device error prints a message on stderr
 * and exits with EXIT_FAILURE (src/hvm.cu:2360-2367).
 */
void hvm_cu(const uint32_t* book_buffer);

/* ---- Front-end ---------------------------------------------------------------
 *
 * Replaces `ast::Book::parse(code).build().to_buffer(&mut buf)`
 * (src/main.rs:87-92; src/ast.rs:44-634; src/hvm.rs:957-1003), which the
 * reference runs in Rust before calling `hvm_cu`.
 * Writes the book buffer into `out` (capacity `out_cap_words` u32 words) and
 * its length into `*out_words`; call with `out == NULL` to query the length.
 * Returns 0, or 1 (parse error), 2 (build error: missing `@main`, unbound
 * reference), 3 (output too small); `err` receives the message.
 */
int hvm_gb300_book_from_text(const char* text, uint32_t* out, size_t out_cap_words,
                             size_t* out_words, char* err, size_t err_cap);

/* Canonical form of one printed tree (the text after "Result:"): variables
 * renamed x0, x1, ... in first-occurrence order and numbers as their 29-bit
 * Numb word, the comparison the reference's test harness makes
 * (tests/run.rs:112-147). Returns 0, 1 on a parse error, 3 if `out` is too
 * small; `out == NULL` queries the length. */
int hvm_gb300_canonical_tree(const char* text, char* out, size_t out_cap, size_t* out_len,
                             char* err, size_t err_cap);

/* CUDA source of the compiled calls for a serialized book (the reference's
 * cmp::compile_book for its CUDA target, src/cmp.rs:10-119, which its gen-cu
 * leaves disabled at src/main.rs:140-146): per def, its node stores and links
 * as straight-line code. `hvm gen-cu --compiled` appends it to the standalone
 * program, which then defines HVM_COMPILED_CALLS. No GPU is used. Returns 0,
 * 1 on a bad book, 3 if `out` is too small; `out == NULL` queries the length
 * (without the terminating NUL). */
int hvm_gb300_compile_calls(const uint32_t* book, size_t words, char* out, size_t out_cap, size_t* out_len,
                            char* err, size_t err_cap);

/* ---- Handle API ----------------------------------------------------------------
 *
 * Re-entrant form of `hvm_cu` for callers that run many nets, read results
 * programmatically, or time the evaluator: it splits the reference's
 * book_load -> gnet_create -> boot -> do_run_io -> print sequence
 * (src/hvm.cu:2320-2397, src/run.cu:857-925) into separate calls.
 */
typedef struct hvm_gb300_runtime hvm_gb300_runtime;

typedef struct {
  int32_t device;             /* CUDA device ordinal */
  uint32_t threads_per_block; /* multiple of 32, at most 128 */
  uint32_t stack_cap;         /* redexes per thread in the shared-memory LIFO */
  uint32_t blocks_per_sm;     /* 0 = as many as fit */
  uint32_t node_log2;         /* node space 2^k words (k <= 29 with 32-bit ports, <= 32 in the 64-bit
                                 port library libhvm_gb300_p64.so) */
  uint32_t vars_log2;         /* var space 2^k words (same bounds) */
  uint32_t ring_log2;         /* global redex ring 2^k entries */
  uint32_t max_turns;         /* 0 = unbounded; else fail after this many turns */
  uint32_t stop_frac_q8;      /* a turn ends once busy threads < (1 - f/256) x initially busy */
  uint32_t trace_cap;         /* record up to this many turns (0 = off), see hvm_gb300_trace */
  uint32_t reg_cap_blocks;    /* 0, or 5/6/8: cap registers so that many 128-thread blocks fit per SM */
  uint32_t profile;           /* 1 = collect per-warp round counters into hvm_gb300_stats.prof (a
                                 separately compiled kernel variant: register caps 0 and 8, no
                                 fast_calls) */
  uint32_t graph_turns;       /* 0 = one launch per turn; k > 0 = turns run as replays of a CUDA
                                 graph of k launches (captured once per loaded book/batch) */
  uint32_t node_page_log2;    /* allocator page of 2^k node words (0 = 9; 5..12) */
  uint32_t var_page_log2;     /* allocator page of 2^k var words (0 = 10; 5..12) */
  uint32_t max_pages;         /* pages a thread may own per space (0 = 2^15 node / 2^16 var words' worth) */
  uint32_t steal_min;         /* a lane gives its oldest redex to an empty lane of its warp once it holds
                                 this many (0 = 2) */
  uint32_t turn_budget_cap;   /* 0, or the most rounds a turn may run (default 1024): bounds how long a
                                 stream waits between admissions and completion checks (serving latency) */
  uint32_t narrow_below;      /* 0 = off; else (default 1024) turns that start with fewer pending redexes
                                 than this run the `narrow_reg_cap` kernel variant on its own grid, the
                                 others the `reg_cap_blocks` one; the host switches between its polls */
  uint32_t narrow_reg_cap;    /* 0 (default: no register cap, no spills), or 5/6/8: the register cap of
                                 that narrow variant */
  uint32_t rule_select;       /* 0 = every lane with a redex interacts each round; 1 (default) = a warp
                                 runs one rule class per round (no allocation: LINK/VOID/ERAS/ANNI; CALL;
                                 COMM; OPER/SWIT), the class of most lanes' next redex, a lane that has
                                 waited 4 rounds going first; 2 = one rule per round */
  uint32_t fast_calls;        /* CALL-time fast paths of the reference's compiled C mode (src/cmp.rs:
                                 110-290), same interaction counts: 0 = off (default); 1 = a def whose
                                 root is `(?((s1 s2) r) r)` called with `(#X R)` switches on the spot;
                                 2 = also, a def whose root is a CON called with a CON annihilates it
                                 on the spot (compiled for register caps 0, 5 and 8) */
  uint32_t local_nets;        /* 1 = block-local nets in shared memory (the reference's LNet + LEAK,
                                 src/hvm.cu:130-135, 1129-1174): fresh words of a turn in the block's
                                 shared memory, copied out to HBM when a global var would point at
                                 them and at the turn's end; 128-thread blocks, register caps 0/8 */
  uint32_t persistent;        /* 1 = a normalisation (single net or batch) runs its turns inside
                                 cooperative launches of up to 4096 turns each, closed on the device
                                 (register caps 0 and 8, no fast_calls/profile/local_nets; streams keep
                                 one launch per turn); 0 = one launch per turn (default) */
  uint32_t upper_half;        /* 1 = the allocator hands out words from the upper half of each space
                                 only (every fresh word has a high index: with 64-bit ports and 2^32-word
                                 spaces, indices beyond the 32-bit port's range) */
} hvm_gb300_config;

typedef struct {
  uint64_t itrs;          /* interactions, counted as the reference counts them */
  uint64_t leak;          /* redexes that went through the global ring */
  uint64_t turns;         /* evaluator turns run */
  uint64_t retries;       /* availability re-tries */
  uint64_t rule_hist[8];  /* interactions per rule: LINK CALL VOID ERAS ANNI COMM OPER SWIT */
  uint64_t prof[8];       /* with profile=1: rounds, busy lanes, link steps, warp cycles in
                             the turn loop, and in the load / write / fence / link phases */
  double seconds;         /* wall time inside normalisation */
  double kernel_ms;       /* device time of the turn kernels (CUDA events around each launch) */
  uint64_t turn_launches; /* turn-kernel launches (including trailing no-op turns) */
  uint64_t launches;      /* all kernel launches of this library */
  uint64_t h2d_bytes;     /* bytes copied host -> device */
  uint64_t d2h_bytes;     /* bytes copied device -> host */
  uint32_t threads, grid, block;
} hvm_gb300_stats;

/* Fills `cfg` with the defaults used by `hvm_cu`. */
void hvm_gb300_default_config(hvm_gb300_config* cfg);

/* Creates a runtime on `cfg->device` (NULL = defaults) and allocates its net.
 * Returns 0; on failure *out may still hold a runtime whose error text says why. */
int hvm_gb300_create(const hvm_gb300_config* cfg, hvm_gb300_runtime** out);

/* Loads a book buffer (`words` = its length in u32, or 0 if unknown). Same
 * limits as the reference's C loader (src/hvm.c:1408-1453). */
int hvm_gb300_load_book(hvm_gb300_runtime* rt, const uint32_t* book_buffer, size_t words);

/* Clears the net, boots `@main ~ ROOT`, normalises, and runs the readback
 * expansion of the IO loop (which can add interactions). `stats` may be NULL. */
int hvm_gb300_run(hvm_gb300_runtime* rt, hvm_gb300_stats* stats);

/* The normal form at ROOT in the reference's printed format (without the
 * "Result: " prefix). `out == NULL` queries the length (excluding the NUL). */
int hvm_gb300_result(hvm_gb300_runtime* rt, char* out, size_t cap, size_t* len);

/* ---- Batches ------------------------------------------------------------------
 *
 * No single counterpart in the reference, which evaluates one net per call
 * (src/hvm.cu:2320): many independent nets are evaluated together by the same
 * launches. Net k keeps its own ROOT var; the total interaction count is the
 * sum of the nets' counts under the reference.
 *
 * hvm_gb300_load_batch: `books[k]` is net k's book buffer (`words[k]` its
 * length, or words == NULL). hvm_gb300_run_batch: boots every net's @main,
 * normalises all of them, runs each net's readback expansion.
 * hvm_gb300_batch_roots: each net's normal-form root port with var chains
 * resolved (a number for numeric results). hvm_gb300_batch_result: one net's
 * normal form as text, like hvm_gb300_result. */
int hvm_gb300_load_batch(hvm_gb300_runtime* rt, const uint32_t* const* books, const size_t* words, uint32_t n);
int hvm_gb300_run_batch(hvm_gb300_runtime* rt, hvm_gb300_stats* stats);
int hvm_gb300_batch_roots(hvm_gb300_runtime* rt, uint32_t* out, size_t cap);

/* Turns the loaded batch into request templates: afterwards the batch has
 * `n` nets, net r being a fresh copy of loaded net templates[r] (sharing its
 * definitions, with its own ROOT). Used to serve many requests of a few
 * programs without loading a book per request. */
int hvm_gb300_set_requests(hvm_gb300_runtime* rt, const uint32_t* templates, uint32_t n);

/* Continuous batching over a loaded batch (serving): net k is admitted once
 * `arrival_s[k]` seconds have passed (non-decreasing), while fewer than
 * `max_inflight` nets are in flight (0 = no cap) and live node and var words
 * stay under `live_frac` of their spaces; admitted nets share the turns with
 * the nets already running. `order` 0 admits arrived nets first come, first
 * served; 1 admits the smallest book first. A net completes when its ROOT becomes a number
 * (`done_s[k]` = seconds since the start, `result_ports[k]` = that port);
 * nets with other normal forms complete when the batch is quiescent. The
 * stats' itrs is the total over all nets. */
int hvm_gb300_run_stream(hvm_gb300_runtime* rt, const double* arrival_s, uint32_t max_inflight, double live_frac,
                         uint32_t order, double* done_s, uint32_t* result_ports, hvm_gb300_stats* stats);
int hvm_gb300_batch_result(hvm_gb300_runtime* rt, uint32_t net, char* out, size_t cap, size_t* len);

/* Diagnostic counterpart of the reference's count_memory kernel
 * (src/hvm.cu:2234-2255): out[0] live node words, out[1] live var words,
 * out[2] node words taken but not yet written, out[3] / out[4] node / var
 * pages handed out by the pools so far. */
int hvm_gb300_count_live(hvm_gb300_runtime* rt, uint64_t* out);

/* One evaluator turn as recorded on the device (no reference counterpart:
 * the reference's per-turn state is only visible through printf debugging,
 * src/hvm.cu:1729-1740). */
typedef struct {
  uint64_t t_ns;        /* device clock when the turn closed */
  int64_t live_nodes;   /* node words in use after the turn */
  uint64_t itrs;        /* cumulative interactions */
  uint64_t pending;     /* redexes left for the next turn */
  uint32_t dry;         /* threads that ran out of work */
  uint32_t stopped;     /* 1 if the turn was ended by the dry rule */
  uint32_t budget;      /* interactions per thread allowed in the turn */
  uint32_t per_thread;  /* input redexes each thread took at the start */
  float features[16];   /* scheduler inputs computed when the turn closed */
  float outputs[3];     /* next turn's budget, stop fraction and static share,
                           in the policy's output space (hvm_gb300_set_policy) */
} hvm_gb300_turn;

/* Copies up to `cap` turn records of the last run (needs trace_cap > 0);
 * `*n` receives how many exist. */
int hvm_gb300_trace(hvm_gb300_runtime* rt, hvm_gb300_turn* out, size_t cap, size_t* n);

/* ---- Turn scheduler -----------------------------------------------------------------
 *
 * Replaces the reference's fixed SEED/GROW/WORK turn policy
 * (src/hvm.cu:1509-1548) for the runtime's later runs. After every turn the
 * scheduler picks three parameters of the next one, each encoded in [0, 1]:
 *   o0  turn budget   64 << round(10 o0) rounds per warp (64 .. 65536)
 *   o1  stop fraction the turn ends once (32 + 192 o1)/256 of the initially
 *                     busy threads have run dry
 *   o2  static share  o2 * min(P/N, cap/2) input redexes per thread at turn
 *                     start when the P pending redexes outnumber the N threads
 * mode HVM_GB300_POLICY_FIXED   the built-in policy (default);
 * mode HVM_GB300_POLICY_LEARNED the MLP 16 -> 64 -> 64 -> 3 (ReLU, sigmoid
 *      outputs) with `weights` packed W1[64][16] b1 W2[64][64] b2 W3[3][64] b3
 *      (HVM_GB300_POLICY_PARAMS floats), evaluated on the device by the turn's
 *      last block from the 16 features of hvm_gb300_turn;
 * mode HVM_GB300_POLICY_CONSTANT `constants[0..2]` while fewer redexes than
 *      threads are pending, `constants[3..5]` otherwise;
 * mode HVM_GB300_POLICY_SCRIPT  per turn: the decision at the close of turn k
 *      is `weights[3k .. 3k+2]` (`n_weights` = 3 x turns; later turns keep the
 *      fixed policy) -- a probe for searching schedules turn by turn.
 * A negative (or non-finite) output keeps the fixed policy's choice. The policy
 * changes only the order of reduction: normal forms and interaction counts are
 * the same under every policy. */
#define HVM_GB300_POLICY_FIXED 0u
#define HVM_GB300_POLICY_LEARNED 1u
#define HVM_GB300_POLICY_CONSTANT 2u
#define HVM_GB300_POLICY_SCRIPT 3u
#define HVM_GB300_POLICY_PARAMS 5443
int hvm_gb300_set_policy(hvm_gb300_runtime* rt, uint32_t mode, const float* weights, size_t n_weights,
                         const float* constants);

/* Policy training (no reference counterpart). Rows of `x` are feature vectors
 * (16 floats), rows of `t` target outputs (3 floats), `sw` per-row weights.
 * The loss is sum_i sw_i * |mlp(x_i) - t_i|^2 / sum_i sw_i.
 *   hvm_gb300_policy_forward  runs the in-kernel inference routine on each row
 *   hvm_gb300_policy_grad     the loss and its gradient (HVM_GB300_POLICY_PARAMS)
 *   hvm_gb300_policy_train    `epochs` full-batch Adam steps (beta 0.9/0.999)
 *                             from `weights`, which receive the result; `loss`
 *                             receives the loss before the last step
 * All run on `device`; return 0, or -1 with `err` set. */
int hvm_gb300_policy_forward(int device, const float* weights, const float* x, size_t n, float* y, char* err,
                             size_t err_cap);
int hvm_gb300_policy_grad(int device, const float* weights, const float* x, const float* t, const float* sw,
                          size_t n, float* grad, float* loss, char* err, size_t err_cap);
int hvm_gb300_policy_train(int device, float* weights, const float* x, const float* t, const float* sw, size_t n,
                           uint32_t epochs, float lr, float* loss, char* err, size_t err_cap);

/* Measures the device's atomic-exchange throughput (no reference counterpart;
 * the denominator of the evaluator's atomic roofline): a full grid issues
 * independent 32-bit atomicExch at pseudo-random addresses of a region of
 * `region_words` (a power of two) words; `*exch_per_s` receives operations per
 * second of device time. Allocates and frees the region. */
int hvm_gb300_atomic_peak(int device, uint64_t region_words, double* exch_per_s, char* err, size_t err_cap);

/* Zeroes the measurement counters of hvm_gb300_stats (kernel_ms, launches,
 * h2d/d2h bytes); they otherwise accumulate over the runtime's life. */
void hvm_gb300_reset_counters(hvm_gb300_runtime* rt);

/* ---- Allocation-free evaluation ---------------------------------------------------
 *
 * No counterpart in the reference. For callers that may not allocate device
 * memory -- a host whose device memory belongs to another allocator or pool,
 * or an embedding that must not fail on allocation -- this evaluates a small
 * net inside one fixed device array of about 20 MB
 * that the library holds on every GPU that loads it, until the process exits.
 * It calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * Limits of the fixed array: book <= 2^19 u32 words, <= 4096 definitions,
 * <= 2^18 node/redex pairs in total, <= 32 nodes and <= 32 vars per
 * definition (the reference CUDA loader's own limit is 64); net <= 2^20 node
 * words and 2^20 var words, at most 8,192 words of each kind per thread of
 * the fixed 2,048-thread grid; at most 2^18 redexes pending at once (the
 * fixed redex ring); normal form <= 2^16 entries. A book beyond the book
 * limits is rejected with a message in `err`; a net that outgrows the memory
 * limits fails with "out of node memory", one that outgrows the ring with
 * "redex ring overflow".
 *
 * Same evaluation as hvm_gb300_run on the current device (boot @main,
 * normalise, readback expansion) without the IO layer: a normal form that
 * asks for an IO call is refused with an error. Its copies, memsets and
 * launches are synchronous calls on the default stream. The normal form is returned breadth-first: out_ports[k]
 * is a port with its var chain resolved; for a node port (CON, DUP, OPR, SWI)
 * its two children are entries out_kids[k] and out_kids[k] + 1 (out_kids is
 * meaningless for other ports). `*out_len` receives the entry count and
 * `*out_itrs` the interaction count. Returns 0, or -1 with `err` set.
 *
 * Every call shares the array: calls that overlap on the GPU race. Each call
 * clears what must start at zero. The first call on a device resolves the
 * array's address with that device current; make it before any stream capture. */
int hvm_gb300_run_noalloc(const uint32_t* book_buffer, size_t words, uint32_t* out_ports, uint32_t* out_kids,
                          size_t out_cap, size_t* out_len, uint64_t* out_itrs, char* err, size_t err_cap);

/* ---- DL_CALL libraries -----------------------------------------------------------
 *
 * An IO program's DL_CALL (handle, symbol, argument) calls `symbol` from a
 * library DL_OPEN loaded as `hvm_gb300_dl_fn` with the net and the argument
 * port, and wraps the port it returns in Ok: the signature of the reference's
 * run-cu, `Port (*)(GNet*, Port)` (src/run.cu:795-813). Ports are the
 * reference's 32-bit words (tag in the low 3 bits). Inside such a call the
 * library reads and extends the device net with the functions below, which
 * replace the host-side net functions run-cu exports (src/hvm.cu:1842-1893,
 * src/run.cu:102-285). Each returns 0, or -1 after recording the error, in
 * which case the DL_CALL, and the run, fail with it.
 */
typedef struct hvm_gb300_io hvm_gb300_io;
typedef uint32_t (*hvm_gb300_dl_fn)(hvm_gb300_io* net, uint32_t arg);

/* Follows substituted vars from `port` and normalises a REF met there
 * (gnet_expand, src/hvm.cu:1871-1882). */
int hvm_gb300_io_expand(hvm_gb300_io* net, uint32_t port, uint32_t* out);
/* The two ports of the node a CON/DUP/OPR/SWI port points to
 * (gnet_node_load, src/hvm.cu:1842-1846). */
int hvm_gb300_io_node_load(hvm_gb300_io* net, uint32_t port, uint32_t* fst, uint32_t* snd);
/* Places a new node (fst, snd) in the net; `*out` = a `tag` port to it
 * (gnet_make_node, src/hvm.cu:1885-1893). */
int hvm_gb300_io_make_node(hvm_gb300_io* net, uint32_t tag, uint32_t fst, uint32_t snd, uint32_t* out);
/* Reads a right-nested tuple of at most `size` elements into `elems`
 * (gnet_readback_tup, src/run.cu:102-117). */
int hvm_gb300_io_readback_tup(hvm_gb300_io* net, uint32_t port, uint32_t size, uint32_t* elems, uint32_t* n);
/* Reads a lambda-encoded list of bytes; `out == NULL` queries the length
 * (gnet_readback_bytes, src/run.cu:124-163). Reading evaluates the list; a
 * length query followed by the read of the same port, with no other net
 * function between them, evaluates it once. */
int hvm_gb300_io_readback_bytes(hvm_gb300_io* net, uint32_t port, uint8_t* out, size_t cap, size_t* len);
/* Places a lambda-encoded list of bytes in the net (gnet_inject_bytes,
 * src/run.cu:267-285). */
int hvm_gb300_io_inject_bytes(hvm_gb300_io* net, const uint8_t* bytes, size_t len, uint32_t* out);

/* Self-test of the bounded wait that persistent launches use between turns
 * (a block waiting for the turn's closing block): one GPU thread waits on a
 * word that nothing writes, with a limit of `limit_ms` (1..10000) of the
 * global timer. `*timed_out` = 1 once the limit ran out (the expected answer)
 * and `*waited_ms` the time it waited. Returns 0, or -1 on a CUDA error. */
int hvm_gb300_wait_probe(int32_t device, uint32_t limit_ms, uint32_t* timed_out, double* waited_ms);

/* Last error message of `rt` ("" if none). */
const char* hvm_gb300_error(const hvm_gb300_runtime* rt);

/* Frees the runtime and its device memory. */
void hvm_gb300_destroy(hvm_gb300_runtime* rt);

#ifdef __cplusplus
}
#endif

#endif /* HVM_GB300_H */
