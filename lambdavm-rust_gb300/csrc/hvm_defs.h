// hvm_defs.h — HVM2 net encodings and the numeric ALU, shared by the host
// (front-end, loader, readback) and the sm_103a evaluator.
//
// Encodings follow the reference bit for bit, because the book buffer, the
// readback and the interaction count must be identical to `hvm run-c`:
//   Port = (val << 3) | tag            src/hvm.c:197-207, src/hvm.cu:281-291
//   Pair = (snd << 32) | fst           src/hvm.c:212-222, src/hvm.cu:294-306
//   Numb = 29-bit word: 5-bit type/op tag + 24-bit payload
//                                      src/hvm.c:354-582, src/hvm.cu:476-688
#pragma once
#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define HVM_HD __host__ __device__ __forceinline__
#else
#define HVM_HD static inline
#endif

// Port width: 32-bit ports (the reference's encoding) by default; a build
// with HVM_PORT64 compiles the evaluator over 64-bit ports and 128-bit node
// pairs. The two builds' symbols live in distinct inline namespaces, so that
// one library can link 32-bit host code (the front-end) beside them.
#ifdef HVM_PORT64
#define HVM_NS_BEGIN namespace hvm { inline namespace p64 {
#else
#define HVM_NS_BEGIN namespace hvm { inline namespace p32 {
#endif
#define HVM_NS_END } }

HVM_NS_BEGIN

typedef uint8_t  Tag;
#ifdef HVM_PORT64
// 64-bit ports: a 61-bit val; a node is a 128-bit pair (fst in the low half).
typedef uint64_t Val;
typedef uint64_t Port;
typedef unsigned __int128 Pair;
constexpr int PORT_BITS = 64;
#else
typedef uint32_t Val;
typedef uint32_t Port;
typedef uint64_t Pair;
constexpr int PORT_BITS = 32;
#endif
typedef uint32_t Numb;
typedef uint8_t  Rule;

// Port tags (src/hvm.c:63-70).
enum : Tag { VAR = 0, REF = 1, ERA = 2, NUM = 3, CON = 4, DUP = 5, OPR = 6, SWI = 7 };

// Interaction rules (src/hvm.c:73-80).
enum : Rule { LINK = 0, CALL = 1, VOID = 2, ERAS = 3, ANNI = 4, COMM = 5, OPER = 6, SWIT = 7 };

// Numb type / operator tags (src/hvm.c:87-109).
enum : uint32_t {
  TY_SYM = 0x00, TY_U24 = 0x01, TY_I24 = 0x02, TY_F24 = 0x03,
  OP_ADD = 0x04, OP_SUB = 0x05, FP_SUB = 0x06, OP_MUL = 0x07,
  OP_DIV = 0x08, FP_DIV = 0x09, OP_REM = 0x0A, FP_REM = 0x0B,
  OP_EQ  = 0x0C, OP_NEQ = 0x0D, OP_LT  = 0x0E, OP_GT  = 0x0F,
  OP_AND = 0x10, OP_OR  = 0x11, OP_XOR = 0x12, OP_SHL = 0x13,
  FP_SHL = 0x14, OP_SHR = 0x15, FP_SHR = 0x16,
};

// Special ports (src/hvm.c:112-114). ROOT is the VAR whose index is 0x1FFFFFFF
// (with 64-bit ports, 0xFFFFFFFF: word indices stay 32-bit, and the ROOT var
// is the last word of any var space either way); NONE is all ones.
#ifdef HVM_PORT64
constexpr Port FREE = 0;
constexpr Val  ROOT_VAR = 0xFFFFFFFFull;
constexpr Port ROOT = ROOT_VAR << 3;
constexpr Port NONE = ~0ull;
#else
constexpr Port FREE = 0x00000000u;
constexpr Port ROOT = 0xFFFFFFF8u;
constexpr Port NONE = 0xFFFFFFFFu;
constexpr Val  ROOT_VAR = 0x1FFFFFFFu;
#endif

// Book limits of the CPU runtime (src/hvm.c:135-136, 161): the GB300 runtime
// accepts exactly what `hvm run-c` accepts, so both reject the same books.
constexpr uint32_t DEF_RBAG_LEN = 0xFFF;
constexpr uint32_t DEF_NODE_LEN = 0xFFF;
constexpr uint32_t MAX_DEFS     = 0x4000;
// Each def header in the buffer: fid, name[64], safe, rbag_len, node_len, vars_len, root.
constexpr uint32_t DEF_HEADER_WORDS = 1 + 64 + 5;

#ifdef HVM_PORT64
// A number keeps the 29-bit Numb a 32-bit port holds: the reference's u24
// arithmetic wraps where (numb << 3) leaves the 32-bit word.
HVM_HD Port new_port(Tag tag, Val val) { return ((tag == NUM ? val & 0x1FFFFFFFull : val) << 3) | tag; }
#else
HVM_HD Port new_port(Tag tag, Val val) { return (val << 3) | tag; }
#endif
HVM_HD Tag  get_tag(Port p) { return (Tag)(p & 7); }
HVM_HD Val  get_val(Port p) { return p >> 3; }
HVM_HD Pair new_pair(Port fst, Port snd) { return ((Pair)snd << PORT_BITS) | fst; }
HVM_HD Port get_fst(Pair p) { return (Port)p; }
HVM_HD Port get_snd(Pair p) { return (Port)(p >> PORT_BITS); }
HVM_HD bool is_nod(Port p) { return get_tag(p) >= CON; }
HVM_HD bool is_var(Port p) { return get_tag(p) == VAR; }

// Par flag: bit 28 of a REF's val in the fst port of a redex (src/hvm.c:224-251).
HVM_HD Pair set_par_flag(Pair p) {
  Port a = get_fst(p);
  return get_tag(a) == REF ? new_pair(new_port(REF, get_val(a) | 0x10000000u), get_snd(p)) : p;
}
HVM_HD bool get_par_flag(Pair p) {
  Port a = get_fst(p);
  return get_tag(a) == REF && (get_val(a) >> 28) == 1;
}

// The 8x8 rule table (src/hvm.c:319-332).
HVM_HD Rule get_rule(Port a, Port b) {
  const Rule t[8][8] = {
    //VAR  REF   ERA   NUM   CON   DUP   OPR   SWI
    {LINK, LINK, LINK, LINK, LINK, LINK, LINK, LINK}, // VAR
    {LINK, VOID, VOID, VOID, CALL, CALL, CALL, CALL}, // REF
    {LINK, VOID, VOID, VOID, ERAS, ERAS, ERAS, ERAS}, // ERA
    {LINK, VOID, VOID, VOID, ERAS, ERAS, OPER, SWIT}, // NUM
    {LINK, CALL, ERAS, ERAS, ANNI, COMM, COMM, COMM}, // CON
    {LINK, CALL, ERAS, ERAS, COMM, ANNI, COMM, COMM}, // DUP
    {LINK, CALL, ERAS, OPER, COMM, COMM, ANNI, COMM}, // OPR
    {LINK, CALL, ERAS, SWIT, COMM, COMM, COMM, ANNI}, // SWI
  };
  return t[get_tag(a)][get_tag(b)];
}
HVM_HD bool should_swap(Port a, Port b) { return get_tag(b) < get_tag(a); }
// LINK, VOID, ERAS, ANNI are "shrinking" rules (src/hvm.c:340-343).
HVM_HD bool is_high_priority(Rule r) { return ((0x1Du >> r) & 1u) != 0; }

// ---- Numb ALU ---------------------------------------------------------------

HVM_HD uint32_t f32_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
HVM_HD float bits_f32(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

HVM_HD Numb new_sym(uint32_t v) { return (v << 5) | TY_SYM; }
HVM_HD uint32_t get_sym(Numb w) { return w >> 5; }
HVM_HD Numb new_u24(uint32_t v) { return (v << 5) | TY_U24; }
HVM_HD uint32_t get_u24(Numb w) { return w >> 5; }
HVM_HD Numb new_i24(int32_t v) { return ((uint32_t)v << 5) | TY_I24; }
HVM_HD int32_t get_i24(Numb w) { return ((int32_t)(w << 3)) >> 8; }
HVM_HD uint32_t get_typ(Numb w) { return w & 0x1F; }

// f24 packing used by the runtimes' ALU (src/hvm.c:373-382). Its rounding
// term uses C's logical `!shifted_bits`, which differs from the parser's
// rounding below on exact ties with an even non-zero mantissa; results of
// `operate` must use this form to match `hvm run-c` bit for bit.
HVM_HD Numb new_f24(float val) {
  uint32_t bits = f32_bits(val);
  uint32_t shifted = bits >> 8;
  uint32_t lost = bits & 0xFF;
  uint32_t nan = (val != val) ? 1u : 0u;
  shifted += (nan ^ 1u) & ((lost - ((lost >> 7) & (shifted == 0 ? 1u : 0u))) >> 7);
  shifted |= nan;
  return (shifted << 5) | TY_F24;
}

// f24 packing used by the `.hvm` parser for literals (src/hvm.rs:257-266):
// the tie term uses Rust's bitwise `!shifted_bits` (round half to even).
HVM_HD Numb new_f24_literal(float val) {
  uint32_t bits = f32_bits(val);
  uint32_t shifted = bits >> 8;
  uint32_t lost = bits & 0xFF;
  uint32_t nan = (val != val) ? 1u : 0u;
  shifted += (nan ^ 1u) & ((lost - ((lost >> 7) & ~shifted)) >> 7);
  shifted |= nan;
  return (shifted << 5) | TY_F24;
}

HVM_HD float get_f24(Numb w) { return bits_f32((w << 3) & 0xFFFFFF00u); }

HVM_HD bool is_num(Numb w) { return get_typ(w) >= TY_U24 && get_typ(w) <= TY_F24; }
HVM_HD bool is_cast(Numb w) { return get_typ(w) == TY_SYM && get_sym(w) >= TY_U24 && get_sym(w) <= TY_F24; }
HVM_HD Numb partial(Numb a, Numb b) { return (b & ~0x1Fu) | get_sym(a); }

HVM_HD float clampf24(float x, float lo, float hi) {
  float t = x < lo ? lo : x;
  return t > hi ? hi : t;
}

// Numeric casts (src/hvm.c:398-436).
HVM_HD Numb cast(Numb a, Numb b) {
  const float U24_MAX = (float)(1 << 24) - 1, U24_MIN = 0.0f;
  const float I24_MAX = (float)(1 << 23) - 1, I24_MIN = (float)(int32_t)((~0u) << 23);
  uint32_t to = get_sym(a), from = get_typ(b);
  if (to == TY_U24) {
    if (from == TY_U24) return b;
    if (from == TY_I24) { int32_t v = get_i24(b); return new_u24((uint32_t)v); }
    if (from == TY_F24) {
      float v = get_f24(b);
      if (v != v) return new_u24(0);
      return new_u24((uint32_t)clampf24(v, U24_MIN, U24_MAX));
    }
  }
  if (to == TY_I24) {
    if (from == TY_U24) { uint32_t v = get_u24(b); return new_i24((int32_t)v); }
    if (from == TY_I24) return b;
    if (from == TY_F24) {
      float v = get_f24(b);
      if (v != v) return new_i24(0);
      return new_i24((int32_t)clampf24(v, I24_MIN, I24_MAX));
    }
  }
  if (to == TY_F24) {
    if (from == TY_U24) return new_f24((float)get_u24(b));
    if (from == TY_I24) return new_f24((float)get_i24(b));
    if (from == TY_F24) return b;
  }
  return new_u24(0);
}

// Binary numeric operation (src/hvm.c:439-558). Integer division or
// remainder by zero is undefined in the reference (SIGFPE on x86); here it
// yields 0 so that a device thread never traps. f24 transcendental cases
// call the platform's math library, as the reference does.
HVM_HD Numb operate(Numb a, Numb b) {
  uint32_t at = get_typ(a), bt = get_typ(b);
  if (at == TY_SYM && bt == TY_SYM) return new_u24(0);
  if (is_cast(a) && is_num(b)) return cast(a, b);
  if (is_cast(b) && is_num(a)) return cast(b, a);
  if (at == TY_SYM && bt != TY_SYM) return partial(a, b);
  if (at != TY_SYM && bt == TY_SYM) return partial(b, a);
  if (at >= OP_ADD && bt >= OP_ADD) return new_u24(0);
  if (at < OP_ADD && bt < OP_ADD) return new_u24(0);
  uint32_t op, ty;
  if (at >= OP_ADD) { op = at; ty = bt; }
  else { op = bt; ty = at; Numb t = a; a = b; b = t; }
  if (ty == TY_U24) {
    uint32_t x = get_u24(a), y = get_u24(b);
    switch (op) {
      case OP_ADD: return new_u24(x + y);
      case OP_SUB: return new_u24(x - y);
      case FP_SUB: return new_u24(y - x);
      case OP_MUL: return new_u24(x * y);
      case OP_DIV: return new_u24(y ? x / y : 0);
      case FP_DIV: return new_u24(x ? y / x : 0);
      case OP_REM: return new_u24(y ? x % y : 0);
      case FP_REM: return new_u24(x ? y % x : 0);
      case OP_EQ:  return new_u24(x == y);
      case OP_NEQ: return new_u24(x != y);
      case OP_LT:  return new_u24(x < y);
      case OP_GT:  return new_u24(x > y);
      case OP_AND: return new_u24(x & y);
      case OP_OR:  return new_u24(x | y);
      case OP_XOR: return new_u24(x ^ y);
      case OP_SHL: return new_u24(x << (y & 31));
      case FP_SHL: return new_u24(y << (x & 31));
      case OP_SHR: return new_u24(x >> (y & 31));
      case FP_SHR: return new_u24(y >> (x & 31));
      default:     return new_u24(0);
    }
  }
  if (ty == TY_I24) {
    int32_t x = get_i24(a), y = get_i24(b);
    // Wrapping arithmetic in uint32 keeps the low 24 bits the reference keeps.
    switch (op) {
      case OP_ADD: return new_i24((int32_t)((uint32_t)x + (uint32_t)y));
      case OP_SUB: return new_i24((int32_t)((uint32_t)x - (uint32_t)y));
      case FP_SUB: return new_i24((int32_t)((uint32_t)y - (uint32_t)x));
      case OP_MUL: return new_i24((int32_t)((uint32_t)x * (uint32_t)y));
      case OP_DIV: return new_i24(y ? x / y : 0);
      case FP_DIV: return new_i24(x ? y / x : 0);
      case OP_REM: return new_i24(y ? x % y : 0);
      case FP_REM: return new_i24(x ? y % x : 0);
      case OP_EQ:  return new_u24(x == y);
      case OP_NEQ: return new_u24(x != y);
      case OP_LT:  return new_u24(x < y);
      case OP_GT:  return new_u24(x > y);
      case OP_AND: return new_i24(x & y);
      case OP_OR:  return new_i24(x | y);
      case OP_XOR: return new_i24(x ^ y);
      default:     return new_i24(0);
    }
  }
  if (ty == TY_F24) {
    float x = get_f24(a), y = get_f24(b);
    switch (op) {
      case OP_ADD: return new_f24(x + y);
      case OP_SUB: return new_f24(x - y);
      case FP_SUB: return new_f24(y - x);
      case OP_MUL: return new_f24(x * y);
      case OP_DIV: return new_f24(x / y);
      case FP_DIV: return new_f24(y / x);
      case OP_REM: return new_f24(fmodf(x, y));
      case FP_REM: return new_f24(fmodf(y, x));
      case OP_EQ:  return new_u24(x == y);
      case OP_NEQ: return new_u24(x != y);
      case OP_LT:  return new_u24(x < y);
      case OP_GT:  return new_u24(x > y);
      case OP_AND: return new_f24(atan2f(x, y));
      case OP_OR:  return new_f24(logf(y) / logf(x));
      case OP_XOR: return new_f24(powf(x, y));
      case OP_SHL: return new_f24((float)sin((double)(x + y)));
      case OP_SHR: return new_f24((float)tan((double)(x + y)));
      default:     return new_f24(0);
    }
  }
  return new_u24(0);
}

HVM_NS_END
