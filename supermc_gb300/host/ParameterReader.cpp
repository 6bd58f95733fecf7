#include "ParameterReader.h"

#include <cctype>
#include <cstdio>
#include <fstream>

namespace smc {
namespace {

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) a++;
  while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) b--;
  return s.substr(a, b - a);
}

std::string key(const std::string &name) {
  std::string k = trim(name);
  for (char &ch : k) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  return k;
}

}  // namespace

void ParameterReader::phraseOneLine(const std::string &line, const std::string &comment) {
  const std::string body = line.substr(0, line.find(comment));
  if (trim(body).empty()) return;
  const size_t eq = body.find('=');
  if (eq == std::string::npos)
    throw ParameterError("\"=\" symbol not found in equation assignment " + body);
  const std::string rhs = trim(body.substr(eq + 1));
  size_t used = 0;
  double v = 0;
  try {
    v = std::stod(rhs, &used);
  } catch (const std::exception &) {
    throw ParameterError("cannot convert \"" + rhs + "\" for " + key(body.substr(0, eq)));
  }
  setVal(body.substr(0, eq), v);
}

void ParameterReader::readFromFile(const std::string &filename, const std::string &comment) {
  std::ifstream f(filename);
  if (!f) throw ParameterError("file " + filename + " does not exist");
  std::string line;
  while (std::getline(f, line)) phraseOneLine(line, comment);
}

void ParameterReader::readFromArguments(long argc, char *argv[], const std::string &comment, long start_from) {
  for (long i = start_from; i < argc; i++) phraseOneLine(argv[i], comment);
}

bool ParameterReader::exist(const std::string &name) const { return values_.count(key(name)) != 0; }

void ParameterReader::setVal(const std::string &name, double value) { values_[key(name)] = value; }

double ParameterReader::getVal(const std::string &name) const {
  auto it = values_.find(key(name));
  if (it == values_.end()) throw ParameterError("parameter " + key(name) + " not found");
  return it->second;
}

double ParameterReader::getVal(const std::string &name, double fallback) const {
  auto it = values_.find(key(name));
  return it == values_.end() ? fallback : it->second;
}

void ParameterReader::echo() const {
  for (const auto &kv : values_) std::printf("%s = %g\n", kv.first.c_str(), kv.second);
}

}  // namespace smc
