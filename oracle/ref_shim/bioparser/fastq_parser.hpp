// bioparser/fastq_parser.hpp - stand-in for bioparser 3.0.13's FASTQ
// parser (TEST INFRASTRUCTURE ONLY, see parser.hpp).  A record is an '@'
// header, sequence lines up to a '+' line, then quality lines until the
// quality is as long as the sequence; unequal lengths, a missing name or
// an empty sequence make an invalid file.
#ifndef ORACLE_SHIM_BIOPARSER_FASTQ_PARSER_HPP_
#define ORACLE_SHIM_BIOPARSER_FASTQ_PARSER_HPP_

#include "bioparser/parser.hpp"

namespace bioparser {

template <class T>
class FastqParser : public Parser<T> {
 public:
  explicit FastqParser(gzFile f) : Parser<T>(f) {}

  std::vector<std::unique_ptr<T>> Parse(std::uint64_t,
                                        bool shorten_names = true) override {
    std::vector<std::unique_ptr<T>> out;
    std::string line;
    while (this->Line(&line)) {
      if (line.empty()) continue;
      if (line[0] != '@') Invalid();
      const std::string name = this->Name(line, shorten_names);
      std::string data, quality;
      bool plus = false;
      while (this->Line(&line)) {
        if (!line.empty() && line[0] == '+') {
          plus = true;
          break;
        }
        data += line;
      }
      if (!plus) Invalid();
      while (quality.size() < data.size() && this->Line(&line)) quality += line;
      if (name.empty() || data.empty() || quality.size() != data.size()) Invalid();
      out.emplace_back(new T(name.c_str(), name.size(), data.c_str(), data.size(),
                             quality.c_str(), quality.size()));
    }
    return out;
  }

 private:
  [[noreturn]] static void Invalid() {
    throw std::invalid_argument("[bioparser::FastqParser] error: invalid file format");
  }
};

}  // namespace bioparser

#endif  // ORACLE_SHIM_BIOPARSER_FASTQ_PARSER_HPP_
