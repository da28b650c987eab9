/* ref_driver.c — test infrastructure only.
 *
 * Entry point for the reference's own C runtime, compiled in place from the
 * reference sources (src/run.c, which includes src/hvm.c) by oracle/Makefile
 * into oracle/_ref/hvm_ref. It does what `hvm run-c` does after the Rust
 * front-end (src/main.rs:74-86): hand the serialized book buffer to
 * `hvm_c(u32*)` (src/hvm.c:1743). The buffer is read from the file named on
 * the command line, as produced by this repository's front-end.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

void hvm_c(uint32_t* book_buffer);

int main(int argc, char** argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: %s <book.bin>\n", argv[0]);
    return 2;
  }
  FILE* f = fopen(argv[1], "rb");
  if (!f) { perror(argv[1]); return 2; }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  uint32_t* buf = (uint32_t*)malloc((size_t)n + 4);
  if (!buf || fread(buf, 1, (size_t)n, f) != (size_t)n) { fprintf(stderr, "read failed\n"); return 2; }
  fclose(f);
  hvm_c(buf);
  free(buf);
  return 0;
}
