/* A library for the DL_CALL parity tests. Every function exists twice, with
 * names of the same length so that the two programs calling them evaluate
 * alike:
 *   *_c  the reference C runtime's signature, Port fn(Net*, Book*, Port)
 *        (src/run.c:681-698), using the net functions of the reference
 *        binary (readback_bytes / inject_bytes, src/run.c:123-161, 224-246;
 *        binary built with -rdynamic, oracle/Makefile ref-dl, so that this
 *        library sees them);
 *   *_g  the GB300 runtime's hvm_gb300_dl_fn, using hvm_gb300_io_*.
 * The golden script runs the *_c programs through the reference binary, the
 * GPU tests the *_g programs through `hvm run-cu`.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "hvm_gb300.h"

/* Each process defines only its own runtime's net functions: the other set
 * stays unresolved (weak), so that the library loads in both. */
#pragma weak hvm_gb300_io_expand
#pragma weak hvm_gb300_io_node_load
#pragma weak hvm_gb300_io_make_node
#pragma weak hvm_gb300_io_readback_tup
#pragma weak hvm_gb300_io_readback_bytes
#pragma weak hvm_gb300_io_inject_bytes

/* Port = (val << 3) | tag with NUM = 3; a u24 Numb = (value << 5) | 1. */
static uint32_t succ_u24(uint32_t port) {
  if ((port & 7u) != 3u || ((port >> 3) & 31u) != 1u) return port;
  const uint32_t v = ((port >> 8) + 1u) & 0xFFFFFFu;
  return (((v << 5) | 1u) << 3) | 3u;
}

uint32_t inc_c(void* net, void* book, uint32_t arg) { (void)net; (void)book; return succ_u24(arg); }
uint32_t inc_g(hvm_gb300_io* net, uint32_t arg) { (void)net; return succ_u24(arg); }

/* The reference C runtime's byte list (src/run.c:27-30) and its two net
 * functions, resolved in the reference binary. */
typedef struct { uint32_t len; char* buf; } RefBytes;
extern RefBytes readback_bytes(void* net, void* book, uint32_t port) __attribute__((weak));
extern uint32_t inject_bytes(void* net, RefBytes* bytes) __attribute__((weak));

static const char GREETING[] = "hi, ";

uint32_t greet_c(void* net, void* book, uint32_t arg) {
  RefBytes in = readback_bytes(net, book, arg);
  RefBytes out;
  out.len = (uint32_t)strlen(GREETING) + in.len;
  out.buf = (char*)malloc(out.len + 1);
  memcpy(out.buf, GREETING, strlen(GREETING));
  memcpy(out.buf + strlen(GREETING), in.buf, in.len);
  free(in.buf);
  const uint32_t r = inject_bytes(net, &out);
  free(out.buf);
  return r;
}

uint32_t greet_g(hvm_gb300_io* net, uint32_t arg) {
  size_t len = 0;
  if (hvm_gb300_io_readback_bytes(net, arg, NULL, 0, &len)) return 0;
  uint8_t* buf = (uint8_t*)malloc(strlen(GREETING) + len + 1);
  memcpy(buf, GREETING, strlen(GREETING));
  uint32_t r = 0;
  if (hvm_gb300_io_readback_bytes(net, arg, buf + strlen(GREETING), len, &len) == 0)
    hvm_gb300_io_inject_bytes(net, buf, strlen(GREETING) + len, &r);
  free(buf);
  return r;
}

/* The pair (arg, arg + 1) as one new CON node, checked back through the
 * tuple and node readbacks: exercises the remaining GB300 net functions. The
 * reference binary exports no node constructor for a library to call, so
 * this one has no C twin; its test compares with a known answer. */
uint32_t two_g(hvm_gb300_io* net, uint32_t arg) {
  uint32_t a = 0, out = 0;
  if (hvm_gb300_io_expand(net, arg, &a)) return 0;
  if (hvm_gb300_io_make_node(net, 4u /* CON */, a, succ_u24(a), &out)) return 0;
  uint32_t elems[2], n = 0;
  if (hvm_gb300_io_readback_tup(net, out, 2, elems, &n) || n != 2 || elems[0] != a) return 0;
  uint32_t fst = 0, snd = 0;
  if (hvm_gb300_io_node_load(net, out, &fst, &snd) || fst != a || snd != succ_u24(a)) return 0;
  return out;
}
