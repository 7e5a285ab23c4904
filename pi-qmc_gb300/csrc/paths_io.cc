// Path files in pi-qmc's restart format: what WritePaths writes
// (src/algorithm/WritePaths.cc:25-114) and PathReader reads
// (src/algorithm/PathReader.cc:20-140), for one serial clone in 3-d.
//
//   #Permutations p0 p1 ... p(N-1)
//   #Path coordinates: N particles in 3-d
//   x y z x y z ...        one line per slice, particle 0 first
//
// Coordinates are printed with 15 significant digits (the stream's
// precision(15) with no float field set, i.e. printf's %.15g), each followed
// by one space.  The host layout is the engine's: [slice][particle][xyz].
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pimc_gb300.h"

namespace pimc {
int set_error(int code, const std::string& msg);  // engine.cu
}

namespace {

// Whitespace-separated tokens of a text file, read the way an istream's >>
// splits them.
struct Tokens {
  std::string text;
  size_t pos = 0;
  bool next(std::string& tok) {
    while (pos < text.size() && isspace((unsigned char)text[pos])) ++pos;
    if (pos >= text.size()) return false;
    const size_t b = pos;
    while (pos < text.size() && !isspace((unsigned char)text[pos])) ++pos;
    tok.assign(text, b, pos - b);
    return true;
  }
  // Rest of the current line (getline), newline consumed.
  void skip_line() {
    while (pos < text.size() && text[pos] != '\n') ++pos;
    if (pos < text.size()) ++pos;
  }
};

bool read_file(const char* filename, std::string& out) {
  FILE* f = fopen(filename, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
  const bool ok = !ferror(f);
  fclose(f);
  return ok;
}

// istream >> double accepts what strtod accepts for a decimal number; a
// non-number or a non-finite value ends the read.
bool parse_double(const std::string& tok, double& v) {
  if (tok.empty()) return false;
  const char c = tok[0];
  if (!(isdigit((unsigned char)c) || c == '-' || c == '+' || c == '.')) return false;
  errno = 0;
  char* end = nullptr;
  v = strtod(tok.c_str(), &end);
  return end == tok.c_str() + tok.size() && std::isfinite(v);
}

bool parse_int(const std::string& tok, long& v) {
  if (tok.empty()) return false;
  char* end = nullptr;
  v = strtol(tok.c_str(), &end, 10);
  return end == tok.c_str() + tok.size();
}

}  // namespace

extern "C" int pimc_paths_write_file(const char* filename, const double* xyz, int npart,
                                     int nslice) {
  if (!filename || !xyz || npart <= 0 || nslice <= 0)
    return pimc::set_error(PIMC_ERR_INVALID, "bad argument");
  std::string out;
  out.reserve((size_t)npart * nslice * 3 * 24 + 128);
  char buf[64];
  // The engine samples no permutations: the global permutation is the identity.
  out += "#Permutations ";
  for (int i = 0; i < npart; ++i) {
    snprintf(buf, sizeof buf, "%d ", i);
    out += buf;
  }
  out += "\n";
  snprintf(buf, sizeof buf, "#Path coordinates: %d particles in 3-d\n", npart);
  out += buf;
  for (int t = 0; t < nslice; ++t) {
    const double* row = xyz + (size_t)t * npart * 3;
    for (int k = 0; k < 3 * npart; ++k) {
      snprintf(buf, sizeof buf, "%.15g ", row[k]);
      out += buf;
    }
    out += "\n";
  }
  FILE* f = fopen(filename, "wb");
  if (!f) return pimc::set_error(PIMC_ERR_INVALID, std::string("cannot open ") + filename);
  const bool ok = fwrite(out.data(), 1, out.size(), f) == out.size();
  if (fclose(f) != 0 || !ok)
    return pimc::set_error(PIMC_ERR_INVALID, std::string("cannot write ") + filename);
  return PIMC_OK;
}

extern "C" int pimc_paths_read_file(const char* filename, double* xyz, int npart, int nslice,
                                    int bfactor) {
  if (!filename || !xyz || npart <= 0 || nslice <= 0 || bfactor <= 0 || nslice % bfactor)
    return pimc::set_error(PIMC_ERR_INVALID, "bad argument");
  Tokens in;
  if (!read_file(filename, in.text))
    return pimc::set_error(PIMC_ERR_INVALID, std::string("cannot read ") + filename);
  const int nfslice = nslice / bfactor;
  std::string tok;
  if (!in.next(tok)) return pimc::set_error(PIMC_ERR_INVALID, "empty path file");
  std::vector<long> perm(npart);
  for (int i = 0; i < npart; ++i) perm[i] = i;
  const bool has_perm = tok == "#Permutations";
  if (has_perm) {
    for (int i = 0; i < npart; ++i)
      if (!in.next(tok) || !parse_int(tok, perm[i]))
        return pimc::set_error(PIMC_ERR_INVALID, "bad #Permutations line");
    in.skip_line();
    if (!in.next(tok)) return pimc::set_error(PIMC_ERR_INVALID, "no coordinates");
  }
  in.skip_line();  // rest of the "#Path coordinates" header
  // nfslice slices (one more, the wrapped first slice, without a permutation line)
  const int nread = nfslice + (has_perm ? 0 : 1);
  std::vector<double> file((size_t)nread * npart * 3);
  for (size_t k = 0; k < file.size(); ++k) {
    if (!in.next(tok) || !parse_double(tok, file[k])) {
      char msg[128];
      snprintf(msg, sizeof msg, "path file ends or is malformed in slice %d of %d",
               (int)(k / (3 * npart)), nread);
      return pimc::set_error(PIMC_ERR_INVALID, msg);
    }
  }
  if (!has_perm) {
    // PathReader matches the wrapped slice to the first slice (sum of |d| < 1e-5).
    const double* wrap = file.data() + (size_t)nfslice * npart * 3;
    for (int i = 0; i < npart; ++i)
      for (int j = 0; j < npart; ++j) {
        double s = 0;
        for (int d = 0; d < 3; ++d) s += std::fabs(wrap[3 * i + d] - file[3 * j + d]);
        if (s < 10e-6) perm[i] = j;
      }
  }
  for (int i = 0; i < npart; ++i)
    if (perm[i] != i)
      return pimc::set_error(PIMC_ERR_INVALID,
                             "path file holds a permutation; the engine samples unpermuted paths");
  // File slice k fills slices k + ib * nslice / bfactor (a restart at bfactor
  // times the number of slices).
  for (int ib = 0; ib < bfactor; ++ib)
    memcpy(xyz + (size_t)ib * nfslice * npart * 3, file.data(),
           (size_t)nfslice * npart * 3 * sizeof(double));
  return PIMC_OK;
}
