// frontend.h — `.hvm` text -> book buffer (C++ side of the front-end).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace hvm {

// Parses `.hvm` text, builds the Book and serializes it in the reference's
// book-buffer format. Returns 0 on success, 1 on a parse error, 2 on a build
// error (missing @main, unbound reference); `err` holds the message.
int book_from_text(const std::string& text, std::vector<uint32_t>& out, std::string& err);

// Canonical form of one printed tree, for bit-exact readback comparison.
int canonical_tree(const std::string& text, std::string& out, std::string& err);

}  // namespace hvm
