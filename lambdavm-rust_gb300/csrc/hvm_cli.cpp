// hvm_cli.cpp — command-line driver with the reference's `run-cu` and
// `gen-cu` surface (src/main.rs:22-65, 87-96, 128-155):
//   hvm run-cu FILE    parses the `.hvm` file, serializes the Book and calls
//                      the C ABI `hvm_cu(book_buffer)`;
//   hvm gen-cu [--compiled] FILE
//                      prints a standalone CUDA program: this runtime as one
//                      translation unit, the serialized book as `BOOK_BUF`, and
//                      a `main` that runs it (compile it with
//                      `nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17`);
//                      with --compiled, the book's defs are also compiled into
//                      straight-line CALL code (the reference's compile_book for
//                      its CUDA target, src/cmp.rs:10-119);
//   hvm book FILE OUT  writes the serialized book buffer to OUT (the bytes the
//                      reference passes across its C ABI).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "hvm_gb300.h"
#include "standalone_source.inc"  // HVM_STANDALONE_SOURCE, generated by build.py

static std::string read_file(const char* path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    fprintf(stderr, "Unable to read file: %s\n", path);
    exit(1);
  }
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

static std::vector<uint32_t> to_buffer(const std::string& code) {
  size_t words = 0;
  char err[1024];
  int rc = hvm_gb300_book_from_text(code.c_str(), nullptr, 0, &words, err, sizeof err);
  if (rc != 0) {
    fprintf(stderr, "%s\n", err);
    exit(101);
  }
  std::vector<uint32_t> buf(words);
  hvm_gb300_book_from_text(code.c_str(), buf.data(), buf.size(), &words, err, sizeof err);
  return buf;
}

static void usage() {
  fprintf(stderr,
          "HVM2 on GB300\n"
          "usage:\n"
          "  hvm run-cu <file.hvm>       evaluate @main on the GPU\n"
          "  hvm gen-cu [--compiled] <file.hvm>\n"
          "                              print a standalone CUDA program for the file\n"
          "  hvm book <file.hvm> <out>   write the serialized book buffer\n");
  exit(2);
}

int main(int argc, char** argv) {
  if (argc < 3) usage();
  std::string cmd = argv[1];
  if (cmd == "run-cu") {
    std::vector<uint32_t> buf = to_buffer(read_file(argv[2]));
    hvm_cu(buf.data());
    return 0;
  }
  if (cmd == "gen-cu") {
    // Like the reference's gen-cu, the book is embedded as a static buffer and
    // the program's main evaluates it through hvm_cu.
    const bool compiled = std::string(argv[2]) == "--compiled";
    if (compiled && argc < 4) usage();
    const char* path = compiled ? argv[3] : argv[2];
    std::vector<uint32_t> buf = to_buffer(read_file(path));
    std::string calls;
    if (compiled) {
      size_t n = 0;
      char err[1024];
      if (hvm_gb300_compile_calls(buf.data(), buf.size(), nullptr, 0, &n, err, sizeof err) != 0) {
        fprintf(stderr, "%s\n", err);
        exit(101);
      }
      calls.resize(n + 1);
      hvm_gb300_compile_calls(buf.data(), buf.size(), &calls[0], calls.size(), &n, err, sizeof err);
      calls.resize(n);
    }
    printf("// Generated by `hvm gen-cu %s%s`: the GB300 evaluator runtime with an embedded book.\n",
           compiled ? "--compiled " : "", path);
    printf("// Build: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 FILE.cu -o FILE\n\n");
    if (compiled) printf("#define HVM_COMPILED_CALLS 1\n\n");
    fputs(HVM_STANDALONE_SOURCE, stdout);
    fputs(calls.c_str(), stdout);
    printf("\n\nstatic const uint32_t BOOK_BUF[%zu] = {", buf.size());
    for (size_t i = 0; i < buf.size(); i++) printf("%s%s%u", i ? "," : "", i % 16 ? "" : "\n  ", buf[i]);
    printf("\n};\n\nint main() {\n  hvm_cu(BOOK_BUF);\n  return 0;\n}\n");
    return 0;
  }
  if (cmd == "book" && argc == 4) {
    std::vector<uint32_t> buf = to_buffer(read_file(argv[2]));
    FILE* f = fopen(argv[3], "wb");
    if (!f || fwrite(buf.data(), 4, buf.size(), f) != buf.size()) {
      fprintf(stderr, "cannot write %s\n", argv[3]);
      return 1;
    }
    fclose(f);
    return 0;
  }
  usage();
  return 2;
}
