/* ref_driver.c — test infrastructure only.
 *
 * Entry point for the reference's own runtimes, compiled in place from the
 * reference sources by oracle/Makefile:
 *   _ref/hvm_ref     src/run.c (which includes src/hvm.c), entry hvm_c
 *                    (src/hvm.c:1743) -- what `hvm run-c` runs;
 *   _ref/hvm_ref_cu  src/run.cu (which includes src/hvm.cu), entry hvm_cu
 *                    (src/hvm.cu:2320) -- what `hvm run-cu` runs, built with
 *                    -DHVM_ENTRY=hvm_cu -DHVM_WALL.
 * Both do what the Rust front-end does before the call (src/main.rs:74-96):
 * hand the serialized book buffer to the entry point. The buffer is read
 * from the file named on the command line.
 *
 * With HVM_WALL the driver creates the CUDA context first and then prints
 * `- WALL: <s>`, the wall-clock time of the whole entry-point call: the
 * reference's own `- TIME` is clock(), the process's CPU time
 * (src/hvm.cu:2335-2345), which leaves out the time its host thread spends
 * blocked on the GPU.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#ifdef HVM_WALL
#include <cuda_runtime_api.h>
#endif

#ifndef HVM_ENTRY
#define HVM_ENTRY hvm_c
#endif

void HVM_ENTRY(uint32_t* book_buffer);

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
#ifdef HVM_WALL
  cudaFree(0);
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
#endif
  HVM_ENTRY(buf);
#ifdef HVM_WALL
  clock_gettime(CLOCK_MONOTONIC, &t1);
  fflush(stdout);
  printf("- WALL: %.6fs\n", (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec));
#endif
  free(buf);
  return 0;
}
