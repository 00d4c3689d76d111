// bioparser/parser.hpp - stand-in for bioparser 3.0.13's Parser, as the
// reference CLI (src/main.cpp) uses it.
//
// TEST INFRASTRUCTURE ONLY: lets oracle/Makefile compile the reference's
// unmodified src/main.cpp (bioparser is fetched by the reference's CMake
// build and is not part of its tree).  Restated from bioparser's published
// interface and file formats: Create<Format>(path) opens a plain or gzip
// file (std::invalid_argument when it cannot), Parse(bytes,
// shorten_names = true) returns the records; names are cut at the first
// whitespace unless shorten_names is false.
#ifndef ORACLE_SHIM_BIOPARSER_PARSER_HPP_
#define ORACLE_SHIM_BIOPARSER_PARSER_HPP_

#include <zlib.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace bioparser {

template <class T>
class Parser {
 public:
  virtual ~Parser() { gzclose(file_); }

  template <template <class> class P>
  static std::unique_ptr<Parser<T>> Create(const std::string& path) {
    gzFile f = gzopen(path.c_str(), "r");
    if (f == nullptr) {
      throw std::invalid_argument(
          "[bioparser::Parser::Create] error: unable to open file " + path);
    }
    return std::unique_ptr<Parser<T>>(new P<T>(f));
  }

  virtual std::vector<std::unique_ptr<T>> Parse(std::uint64_t bytes,
                                                bool shorten_names = true) = 0;

 protected:
  explicit Parser(gzFile f) : file_(f) {}

  // next line without its line end and trailing whitespace; false at EOF
  bool Line(std::string* out) {
    out->clear();
    int ch;
    bool any = false;
    while ((ch = gzgetc(file_)) != -1) {
      any = true;
      if (ch == '\n') break;
      out->push_back(static_cast<char>(ch));
    }
    while (!out->empty() && (out->back() == ' ' || out->back() == '\t' ||
                             out->back() == '\r')) {
      out->pop_back();
    }
    return any;
  }

  static std::string Name(const std::string& header, bool shorten) {
    std::string n = header.substr(1);
    if (shorten) {
      const auto k = n.find_first_of(" \t");
      if (k != std::string::npos) n.resize(k);
    }
    return n;
  }

  gzFile file_;
  std::string pending_;
  bool has_pending_ = false;
};

}  // namespace bioparser

#endif  // ORACLE_SHIM_BIOPARSER_PARSER_HPP_
