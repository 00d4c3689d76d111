// bioparser/fasta_parser.hpp - stand-in for bioparser 3.0.13's FASTA
// parser (TEST INFRASTRUCTURE ONLY, see parser.hpp).  A record is a '>'
// header line and the data lines up to the next header, concatenated;
// a record without a name or without data is an invalid file.
#ifndef ORACLE_SHIM_BIOPARSER_FASTA_PARSER_HPP_
#define ORACLE_SHIM_BIOPARSER_FASTA_PARSER_HPP_

#include "bioparser/parser.hpp"

namespace bioparser {

template <class T>
class FastaParser : public Parser<T> {
 public:
  explicit FastaParser(gzFile f) : Parser<T>(f) {}

  std::vector<std::unique_ptr<T>> Parse(std::uint64_t,
                                        bool shorten_names = true) override {
    std::vector<std::unique_ptr<T>> out;
    std::string line, name, data;
    bool open = false;
    auto flush = [&]() {
      if (!open) return;
      if (name.empty() || data.empty()) {
        throw std::invalid_argument("[bioparser::FastaParser] error: invalid file format");
      }
      out.emplace_back(new T(name.c_str(), name.size(), data.c_str(), data.size()));
    };
    while (this->Line(&line)) {
      if (line.empty()) continue;
      if (line[0] == '>') {
        flush();
        name = this->Name(line, shorten_names);
        data.clear();
        open = true;
      } else {
        data += line;
      }
    }
    flush();
    return out;
  }
};

}  // namespace bioparser

#endif  // ORACLE_SHIM_BIOPARSER_FASTA_PARSER_HPP_
