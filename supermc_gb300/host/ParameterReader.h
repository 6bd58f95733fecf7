// Parameter reader of the drop-in host program: the reference's
// ParameterReader interface (src/ParameterReader.h:14-31) -- key = value
// lines of parameters.dat, then command-line arguments of the same form,
// names trimmed and case-insensitive, everything after '#' a comment -- with
// exceptions where the reference calls exit() (a missing file, a line
// without '=', an unknown name in getVal).
#pragma once
#include <map>
#include <stdexcept>
#include <string>

namespace smc {

struct ParameterError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

class ParameterReader {
 public:
  // ParameterReader::phraseOneLine (src/ParameterReader.cpp:77-84)
  void phraseOneLine(const std::string &line, const std::string &comment = "#");
  // ParameterReader::readFromFile (:87-104)
  void readFromFile(const std::string &filename, const std::string &comment = "#");
  // ParameterReader::readFromArguments (:107-113), argv[start_from..argc)
  void readFromArguments(long argc, char *argv[], const std::string &comment = "#", long start_from = 1);
  bool exist(const std::string &name) const;
  void setVal(const std::string &name, double value);
  double getVal(const std::string &name) const;
  // getVal, or `fallback` when the name was never set
  double getVal(const std::string &name, double fallback) const;
  void echo() const;

 private:
  std::map<std::string, double> values_;
};

}  // namespace smc
