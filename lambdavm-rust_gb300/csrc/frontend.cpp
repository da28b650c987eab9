// frontend.cpp — the `.hvm` IR front-end: parser, Book builder with safety
// propagation, and the book-buffer serializer.
//
// This restates, in C++, the Rust front-end that `hvm run-cu` runs before it
// crosses into CUDA (src/main.rs:87-92):
//   parser      src/ast.rs:44-230   (grammar; TSPL 0.0.13 primitives, see below)
//   builder     src/ast.rs:432-559  (fid order, DFS node numbering, var numbering)
//   safety      src/ast.rs:571-634  (DUP => unsafe, propagated to dependents)
//   serializer  src/hvm.rs:957-1003 (native-endian u32 buffer)
//
// TSPL 0.0.13 (Cargo.lock:6-7) is not vendored with the reference; its parsing
// primitives are restated from their published behaviour: `skip_trivia` skips
// whitespace and `//` line comments, `parse_name` takes [A-Za-z0-9_./-]+,
// `parse_u64` reads decimal, `0x` hex or `0b` binary digits with `_`
// separators. Every program shipped with the reference parses under these
// rules and reproduces its snapshot through the reference's own C runtime.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "hvm_defs.h"
#include "frontend.h"

namespace hvm {
namespace fe {

struct ParseError {
  std::string msg;
};

enum class TK { Var, Ref, Era, Num, Con, Dup, Opr, Swi };

struct Tree {
  TK kind;
  std::string name;        // Var / Ref
  Numb numb = 0;           // Num
  std::unique_ptr<Tree> fst, snd;
};

struct Redex {
  bool par;
  std::unique_ptr<Tree> fst, snd;
};

struct NetAst {
  std::unique_ptr<Tree> root;
  std::vector<Redex> rbag;
};

class Parser {
 public:
  explicit Parser(const std::string& s) : in(s), i(0) {}

  bool eof() { skip_trivia(); return i >= in.size(); }

  // src/ast.rs:202-226 (parse_book): `@name = net` until EOF; a later
  // definition of the same name replaces an earlier one (BTreeMap insert).
  std::map<std::string, NetAst> parse_book() {
    std::map<std::string, NetAst> defs;
    while (!eof()) {
      consume("@");
      std::string name = parse_name();
      consume("=");
      NetAst net = parse_net();
      defs[name] = std::move(net);
    }
    return defs;
  }

  // src/ast.rs:187-200 (parse_net).
  NetAst parse_net() {
    NetAst net;
    net.root = parse_tree();
    skip_trivia();
    while (peek() == '&') {
      consume("&");
      bool par = false;
      if (peek() == '!') { consume("!"); par = true; }
      Redex r;
      r.par = par;
      r.fst = parse_tree();
      consume("~");
      r.snd = parse_tree();
      net.rbag.push_back(std::move(r));
      skip_trivia();
    }
    return net;
  }

  // src/ast.rs:129-185 (parse_tree).
  std::unique_ptr<Tree> parse_tree() {
    skip_trivia();
    auto t = std::make_unique<Tree>();
    char c = peek();
    if (c == '(' || c == '{') {
      advance();
      t->kind = c == '(' ? TK::Con : TK::Dup;
      t->fst = parse_tree();
      skip_trivia();
      t->snd = parse_tree();
      consume(c == '(' ? ")" : "}");
      return t;
    }
    if (c == '$' || c == '?') {
      advance();
      t->kind = c == '$' ? TK::Opr : TK::Swi;
      consume("(");
      t->fst = parse_tree();
      skip_trivia();
      t->snd = parse_tree();
      consume(")");
      return t;
    }
    if (c == '@') {
      advance();
      t->kind = TK::Ref;
      t->name = parse_name();
      return t;
    }
    if (c == '*') {
      advance();
      t->kind = TK::Era;
      return t;
    }
    if (c != 0 && strchr("0123456789+-[", c)) {
      t->kind = TK::Num;
      t->numb = parse_numb();
      return t;
    }
    t->kind = TK::Var;
    t->name = parse_name();
    return t;
  }

  // src/ast.rs:120-127.
  Numb parse_numb() {
    skip_trivia();
    if (peek() == '[') return parse_numb_sym();
    return parse_numb_lit();
  }

  // src/ast.rs:46-100. Order matters: `<<`/`>>` are tried before `<`/`>`.
  Numb parse_numb_sym() {
    consume("[");
    if (try_consume("u24")) { consume("]"); return new_sym(TY_U24); }
    if (try_consume("i24")) { consume("]"); return new_sym(TY_I24); }
    if (try_consume("f24")) { consume("]"); return new_sym(TY_F24); }
    static const struct { const char* s; uint32_t op; } ops[] = {
      {"+", OP_ADD}, {"-", OP_SUB}, {":-", FP_SUB}, {"*", OP_MUL}, {"/", OP_DIV},
      {":/", FP_DIV}, {"%", OP_REM}, {":%", FP_REM}, {"=", OP_EQ}, {"!", OP_NEQ},
      {"<<", OP_SHL}, {":<<", FP_SHL}, {">>", OP_SHR}, {":>>", FP_SHR}, {"<", OP_LT},
      {">", OP_GT}, {"&", OP_AND}, {"|", OP_OR}, {"^", OP_XOR},
    };
    Numb op = 0;
    bool found = false;
    for (auto& o : ops) {
      if (try_consume(o.s)) { op = new_sym(o.op); found = true; break; }
    }
    if (!found) fail("expected operator symbol");
    skip_trivia();
    Numb num = op;
    if (peek() != ']') num = partial(op, parse_numb_lit());
    consume("]");
    return num;
  }

  // src/ast.rs:102-118: f24 if the literal contains '.', "inf" or "NaN";
  // i24 if it starts with a sign; u24 otherwise.
  Numb parse_numb_lit() {
    size_t ini = i;
    while (i < in.size() && (isalnum((unsigned char)in[i]) || in[i] == '+' || in[i] == '-' || in[i] == '.')) i++;
    std::string num = in.substr(ini, i - ini);
    if (num.find('.') != std::string::npos || num.find("inf") != std::string::npos ||
        num.find("NaN") != std::string::npos) {
      float val;
      if (!parse_f32(num, &val)) fail("invalid number literal: " + num);
      return new_f24_literal(val);
    }
    if (!num.empty() && (num[0] == '+' || num[0] == '-')) {
      uint64_t v = parse_u64_str(num, 1);
      int32_t iv = (int32_t)v;
      return new_i24(num[0] == '-' ? (int32_t)(0u - (uint32_t)iv) : iv);
    }
    uint64_t v = parse_u64_str(num, 0);
    return new_u24((uint32_t)v);
  }

  std::string parse_name() {
    skip_trivia();
    size_t ini = i;
    while (i < in.size() && is_name_char(in[i])) i++;
    if (i == ini) fail("expected name");
    return in.substr(ini, i - ini);
  }

  void skip_trivia() {
    while (i < in.size()) {
      char c = in[i];
      if (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v') { i++; continue; }
      if (c == '/' && i + 1 < in.size() && in[i + 1] == '/') {
        while (i < in.size() && in[i] != '\n') i++;
        continue;
      }
      break;
    }
  }

  size_t pos() const { return i; }

 private:
  const std::string& in;
  size_t i;

  static bool is_name_char(char c) {
    return isalnum((unsigned char)c) || c == '_' || c == '.' || c == '-' || c == '/';
  }

  char peek() { return i < in.size() ? in[i] : 0; }
  void advance() { if (i < in.size()) i++; }

  bool try_consume(const char* s) {
    size_t n = strlen(s);
    if (in.compare(i, n, s) == 0) { i += n; return true; }
    return false;
  }

  void consume(const char* s) {
    skip_trivia();
    if (!try_consume(s)) fail(std::string("expected '") + s + "'");
  }

  [[noreturn]] void fail(const std::string& msg) {
    size_t line = 1, col = 1;
    for (size_t k = 0; k < i && k < in.size(); k++) {
      if (in[k] == '\n') { line++; col = 1; } else { col++; }
    }
    throw ParseError{"parse error at line " + std::to_string(line) + ", column " +
                     std::to_string(col) + ": " + msg};
  }

  // TSPL parse_u64 restated: optional 0x/0b prefix, digits with '_' separators;
  // parsing stops at the first non-digit (trailing characters are ignored).
  uint64_t parse_u64_str(const std::string& s, size_t k) {
    unsigned radix = 10;
    if (s.compare(k, 2, "0x") == 0) { radix = 16; k += 2; }
    else if (s.compare(k, 2, "0b") == 0) { radix = 2; k += 2; }
    uint64_t v = 0;
    size_t digits = 0;
    for (; k < s.size(); k++) {
      char c = s[k];
      if (c == '_') continue;
      int d;
      if (c >= '0' && c <= '9') d = c - '0';
      else if (c >= 'a' && c <= 'f') d = c - 'a' + 10;
      else if (c >= 'A' && c <= 'F') d = c - 'A' + 10;
      else break;
      if ((unsigned)d >= radix) break;
      v = v * radix + (uint64_t)d;
      digits++;
    }
    if (digits == 0) fail("expected numeric digit");
    return v;
  }

  // Rust's f32::from_str accepts an optional sign, decimal digits with an
  // optional fraction and exponent, and inf/infinity/nan in any case.
  static bool parse_f32(const std::string& s, float* out) {
    size_t k = 0;
    bool neg = false;
    if (k < s.size() && (s[k] == '+' || s[k] == '-')) { neg = s[k] == '-'; k++; }
    std::string rest = s.substr(k);
    std::string low;
    for (char c : rest) low += (char)tolower((unsigned char)c);
    if (low == "inf" || low == "infinity") { *out = neg ? -INFINITY : INFINITY; return true; }
    if (low == "nan") { *out = neg ? -NAN : NAN; return true; }
    for (char c : rest) {
      if (!(isdigit((unsigned char)c) || c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-')) return false;
    }
    if (rest.empty()) return false;
    char* end = nullptr;
    float v = strtof(s.c_str(), &end);
    if (end != s.c_str() + s.size()) return false;
    *out = v;
    return true;
  }
};

// ---- Builder ---------------------------------------------------------------

struct Def {
  std::string name;
  bool safe = true;
  Port root = 0;
  std::vector<Pair> rbag;
  std::vector<Pair> node;
  uint32_t vars = 0;
};

struct BuildError {
  std::string msg;
};

// src/ast.rs:432-503 (Tree::build): nodes numbered in DFS pre-order with the
// parent's slot reserved first; vars numbered by first occurrence.
static Port build_tree(const Tree& t, Def& def, const std::map<std::string, Val>& fids,
                       std::map<std::string, Val>& vars) {
  switch (t.kind) {
    case TK::Var: {
      auto it = vars.find(t.name);
      if (it == vars.end()) {
        Val v = (Val)vars.size();
        vars[t.name] = v;
        def.vars += 1;
        return new_port(VAR, v);
      }
      return new_port(VAR, it->second);
    }
    case TK::Ref: {
      auto it = fids.find(t.name);
      if (it == fids.end()) throw BuildError{"Unbound definition: " + t.name};
      return new_port(REF, it->second);
    }
    case TK::Era:
      return new_port(ERA, 0);
    case TK::Num:
      return new_port(NUM, t.numb);
    default: {
      Tag tag = t.kind == TK::Con ? CON : t.kind == TK::Dup ? DUP : t.kind == TK::Opr ? OPR : SWI;
      if (t.kind == TK::Dup) def.safe = false;
      size_t index = def.node.size();
      def.node.push_back(0);
      Port p1 = build_tree(*t.fst, def, fids, vars);
      Port p2 = build_tree(*t.snd, def, fids, vars);
      def.node[index] = new_pair(p1, p2);
      return new_port(tag, (Val)index);
    }
  }
}

static void collect_refs(const Tree& t, std::set<std::string>& acc) {
  if (t.kind == TK::Ref) acc.insert(t.name);
  if (t.fst) collect_refs(*t.fst, acc);
  if (t.snd) collect_refs(*t.snd, acc);
}

// src/ast.rs:528-634 (Book::build + propagate_safety).
static std::vector<Def> build_book(const std::map<std::string, NetAst>& defs) {
  std::map<std::string, Val> name_to_fid;
  std::vector<std::string> fid_to_name;
  name_to_fid["main"] = 0;
  fid_to_name.push_back("main");
  for (auto& kv : defs) {
    if (kv.first != "main") {
      name_to_fid[kv.first] = (Val)fid_to_name.size();
      fid_to_name.push_back(kv.first);
    }
  }
  std::vector<Def> book;
  for (auto& name : fid_to_name) {
    auto it = defs.find(name);
    if (it == defs.end()) throw BuildError{"missing `@main` definition"};
    Def def;
    def.name = name;
    std::map<std::string, Val> vars;
    const NetAst& net = it->second;
    def.root = build_tree(*net.root, def, name_to_fid, vars);
    for (auto& r : net.rbag) {
      size_t index = def.rbag.size();
      def.rbag.push_back(0);
      Port p1 = build_tree(*r.fst, def, name_to_fid, vars);
      Port p2 = build_tree(*r.snd, def, name_to_fid, vars);
      Pair rx = new_pair(p1, p2);
      def.rbag[index] = r.par ? set_par_flag(rx) : rx;
    }
    book.push_back(std::move(def));
  }
  // Dependents: B -> {A : A references B}.
  std::map<std::string, std::set<std::string>> dependents;
  for (auto& kv : defs) dependents[kv.first];
  for (auto& kv : defs) {
    std::set<std::string> deps;
    collect_refs(*kv.second.root, deps);
    for (auto& r : kv.second.rbag) { collect_refs(*r.fst, deps); collect_refs(*r.snd, deps); }
    for (auto& d : deps) dependents[d].insert(kv.first);
  }
  std::vector<std::string> stack;
  for (auto& kv : defs) {
    if (!book[name_to_fid[kv.first]].safe) {
      for (auto& n : dependents[kv.first]) stack.push_back(n);
    }
  }
  while (!stack.empty()) {
    std::string cur = stack.back();
    stack.pop_back();
    Def& d = book[name_to_fid[cur]];
    if (!d.safe) continue;
    d.safe = false;
    for (auto& n : dependents[cur]) stack.push_back(n);
  }
  return book;
}

// src/hvm.rs:957-1003 (Book::to_buffer).
static std::vector<uint32_t> serialize(const std::vector<Def>& book) {
  std::vector<uint32_t> buf;
  buf.push_back((uint32_t)book.size());
  for (size_t fid = 0; fid < book.size(); fid++) {
    const Def& d = book[fid];
    buf.push_back((uint32_t)fid);
    if (d.name.size() >= 256) throw BuildError{"Name too long: " + d.name};
    uint32_t name[64];
    memset(name, 0, sizeof(name));
    memcpy(name, d.name.data(), d.name.size());
    buf.insert(buf.end(), name, name + 64);
    buf.push_back(d.safe ? 1u : 0u);
    buf.push_back((uint32_t)d.rbag.size());
    buf.push_back((uint32_t)d.node.size());
    buf.push_back(d.vars);
    buf.push_back(d.root);
    for (Pair p : d.rbag) { buf.push_back((uint32_t)p); buf.push_back((uint32_t)(p >> 32)); }
    for (Pair p : d.node) { buf.push_back((uint32_t)p); buf.push_back((uint32_t)(p >> 32)); }
  }
  return buf;
}

}  // namespace fe

int book_from_text(const std::string& text, std::vector<uint32_t>& out, std::string& err) {
  try {
    fe::Parser p(text);
    auto defs = p.parse_book();
    auto book = fe::build_book(defs);
    out = fe::serialize(book);
    return 0;
  } catch (const fe::ParseError& e) {
    err = e.msg;
    return 1;
  } catch (const fe::BuildError& e) {
    err = e.msg;
    return 2;
  }
}

// Parses one tree (the text after `Result:`) into a canonical form used to
// compare readbacks: variables renamed x0, x1, ... by first occurrence and
// numbers printed as their 29-bit Numb word, which makes f24 values compare
// bit for bit regardless of how they were formatted (src/tests/run.rs:112-147
// normalises the same way through the Rust parser).
namespace fe {
static void canon(const Tree& t, std::map<std::string, size_t>& vars, std::string& out) {
  switch (t.kind) {
    case TK::Var: {
      auto it = vars.find(t.name);
      size_t k;
      if (it == vars.end()) { k = vars.size(); vars[t.name] = k; } else { k = it->second; }
      out += "x" + std::to_string(k);
      return;
    }
    case TK::Ref: out += "@" + t.name; return;
    case TK::Era: out += "*"; return;
    case TK::Num: {
      char b[32];
      snprintf(b, sizeof b, "#%07X", t.numb & 0x1FFFFFFFu);
      out += b;
      return;
    }
    default: {
      const char* open = t.kind == TK::Con ? "(" : t.kind == TK::Dup ? "{" : t.kind == TK::Opr ? "$(" : "?(";
      const char* close = t.kind == TK::Dup ? "}" : ")";
      out += open;
      canon(*t.fst, vars, out);
      out += " ";
      canon(*t.snd, vars, out);
      out += close;
      return;
    }
  }
}
}  // namespace fe

int canonical_tree(const std::string& text, std::string& out, std::string& err) {
  try {
    fe::Parser p(text);
    auto t = p.parse_tree();
    std::map<std::string, size_t> vars;
    out.clear();
    fe::canon(*t, vars, out);
    return 0;
  } catch (const fe::ParseError& e) {
    err = e.msg;
    return 1;
  }
}

}  // namespace hvm

// ---- C ABI -------------------------------------------------------------------

static void copy_err(const std::string& e, char* err, size_t cap) {
  if (!err || cap == 0) return;
  size_t n = e.size() < cap - 1 ? e.size() : cap - 1;
  memcpy(err, e.data(), n);
  err[n] = 0;
}

extern "C" int hvm_gb300_book_from_text(const char* text, uint32_t* out, size_t out_cap_words,
                                        size_t* out_words, char* err, size_t err_cap) {
  std::vector<uint32_t> buf;
  std::string e;
  int rc = hvm::book_from_text(text ? std::string(text) : std::string(), buf, e);
  if (rc != 0) { copy_err(e, err, err_cap); return rc; }
  if (out_words) *out_words = buf.size();
  if (out && out_cap_words >= buf.size()) memcpy(out, buf.data(), buf.size() * 4);
  else if (out) { copy_err("output buffer too small", err, err_cap); return 3; }
  return 0;
}

extern "C" int hvm_gb300_canonical_tree(const char* text, char* out, size_t out_cap, size_t* out_len,
                                        char* err, size_t err_cap) {
  std::string s, e;
  int rc = hvm::canonical_tree(text ? std::string(text) : std::string(), s, e);
  if (rc != 0) { copy_err(e, err, err_cap); return rc; }
  if (out_len) *out_len = s.size();
  if (out && out_cap > s.size()) { memcpy(out, s.data(), s.size()); out[s.size()] = 0; }
  else if (out) { copy_err("output buffer too small", err, err_cap); return 3; }
  return 0;
}
