// list_reader.h - Fortran list-directed READ semantics for the reference's
// data files: each READ starts a new record, takes as many values as it needs
// across records and drops the rest of its last record.  Separators are
// blanks, tabs and commas; '!' or '/' ends the useful part of a record.
// Numbers follow Fortran input rules: a 'd'/'D' exponent letter, or none at
// all when the exponent is signed ("2.066-1" reads as 0.2066).
#pragma once
#include <cstdlib>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace mcx {

class ListReader {
 public:
  explicit ListReader(const std::string& path) : path_(path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("can't open data file " + path);
    std::string l;
    while (std::getline(in, l)) lines_.push_back(l);
  }
  bool eof() const { return pos_ >= lines_.size(); }
  const std::string& path() const { return path_; }

  // One READ of n numbers; returns false at end of file.
  bool read(int n, std::vector<double>& out) {
    out.clear();
    while ((int)out.size() < n) {
      if (pos_ >= lines_.size()) return false;
      tokens(lines_[pos_++], out, n);
    }
    return true;
  }
  std::vector<double> need(int n) {
    std::vector<double> v;
    if (!read(n, v)) throw std::runtime_error("data file truncated: " + path_);
    return v;
  }
  // One READ of n numbers from exactly one record.  Returns 1 on success, 0
  // when the record does not start with n numbers (a READ error: the caller
  // keeps its previous values, as gfortran does), -1 at end of file.
  int readRecord(int n, std::vector<double>& out) {
    if (pos_ >= lines_.size()) return -1;
    std::vector<double> v;
    tokens(lines_[pos_++], v, n);
    if ((int)v.size() < n) return 0;
    out = v;
    return 1;
  }
  // READ with no items / a character item / a formatted A record: skips one record.
  void skip(int n = 1) {
    for (int i = 0; i < n; ++i) {
      if (pos_ >= lines_.size()) throw std::runtime_error("data file truncated: " + path_);
      ++pos_;
    }
  }
  // The raw text of the next record (formatted A read).
  std::string record() {
    if (pos_ >= lines_.size()) throw std::runtime_error("data file truncated: " + path_);
    return lines_[pos_++];
  }
  // One READ of a (possibly quoted) string.
  std::string readString() {
    while (pos_ < lines_.size()) {
      const std::string& l = lines_[pos_++];
      size_t i = l.find_first_not_of(" \t");
      if (i == std::string::npos) continue;
      if (l[i] == '\'' || l[i] == '"') {
        size_t j = l.find(l[i], i + 1);
        return l.substr(i + 1, j == std::string::npos ? std::string::npos : j - i - 1);
      }
      size_t j = l.find_first_of(" \t,", i);
      return l.substr(i, j == std::string::npos ? std::string::npos : j - i);
    }
    throw std::runtime_error("data file truncated: " + path_);
  }

  // Parses one Fortran real; returns false if t is not a number.
  static bool number(const std::string& tok, double& v) {
    std::string t = tok;
    for (auto& c : t) if (c == 'd' || c == 'D') c = 'e';
    char* end = nullptr;
    v = std::strtod(t.c_str(), &end);
    if (end == t.c_str()) return false;
    if (*end == '+' || *end == '-') {       // exponent without its letter
      char* e2 = nullptr;
      long ex = std::strtol(end, &e2, 10);
      if (e2 != end + 1) {
        v = std::strtod((t.substr(0, (size_t)(end - t.c_str())) + "e" + std::to_string(ex)).c_str(), nullptr);
      }
    }
    return true;
  }

 private:
  static void tokens(const std::string& l, std::vector<double>& out, int n) {
    size_t i = 0;
    while (i < l.size() && (int)out.size() < n) {
      while (i < l.size() && (l[i] == ' ' || l[i] == '\t' || l[i] == ',' || l[i] == '\r')) ++i;
      if (i >= l.size() || l[i] == '!' || l[i] == '/') break;
      size_t j = i;
      while (j < l.size() && !(l[j] == ' ' || l[j] == '\t' || l[j] == ',' || l[j] == '\r')) ++j;
      double v;
      if (!number(l.substr(i, j - i), v)) break;   // a non-numeric token ends the useful part
      out.push_back(v);
      i = j;
    }
  }
  std::string path_;
  std::vector<std::string> lines_;
  size_t pos_ = 0;
};

}  // namespace mcx
