// abi_io.cu -- the reference's on-disk formats, host side only.
//
// Three kinds of file cross the boundary between the reference's integral
// phase, its SCF and this library (xchf1_independent/GAM_IO.f):
//   * direct-access integral files (*.ufm): OPEN(...,FORM='unformatted',
//     ACCESS='direct',RECL=8); record ia holds one FP64 at packed index ia.
//     No record markers; each record is `recl` bytes with the value in its
//     first 8 (gfortran counts RECL in bytes -> 8; ifort without
//     -assume byterecl counts 4-byte words -> 32, the rest zero-padded).
//   * formatted MO files (guessC*.inp read with FORMAT(I2,I3,5E15.8),
//     GAM_IO.f:267; FinalC*.dat written by PUSQLF with
//     FORMAT(I2,I3,1P,5E15.8), GAM_IO.f:471-518): for every MO j, rows of
//     five coefficients labelled MOD(j,100), MOD(row,1000).
//   * ENUCRP.dat: one list-directed real (class_nuc_rep.f:39-41,
//     xcscf.f:248-250).
// No function here touches the GPU.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/neoxc.h"
#include "neoxc_internal.h"

namespace {

using neoxc::set_last_error;

long resolve_recl(int64_t recl) {
  if (recl > 0) return (long)recl;
  const char* e = std::getenv("NEOXC_UFM_RECL");
  return e ? std::atol(e) : 8;
}

// One Fortran 1PE15.8 field: d.ddddddddE+xx, or d.dddddddd+xxx when the
// exponent needs three digits (the letter is dropped, as Fortran's Ew.d
// editing does for 99 < |exp| <= 999), right-justified in 15 columns.
void put_e15_8(std::string& out, double v) {
  char buf[64];
  if (std::isnan(v)) {
    std::snprintf(buf, sizeof buf, "%15s", "NaN");
  } else if (std::isinf(v)) {
    std::snprintf(buf, sizeof buf, "%15s", v < 0 ? "-Infinity" : "Infinity");
  } else {
    char m[48];
    std::snprintf(m, sizeof m, "%.8E", v);  // [-]d.ddddddddE[+-]xx[x]
    char* e = std::strchr(m, 'E');
    const int ex = std::atoi(e + 1);
    *e = '\0';
    const int aex = ex < 0 ? -ex : ex;
    char field[48];
    if (aex <= 99)
      std::snprintf(field, sizeof field, "%sE%c%02d", m, ex < 0 ? '-' : '+', aex);
    else
      std::snprintf(field, sizeof field, "%s%c%03d", m, ex < 0 ? '-' : '+', aex);
    std::snprintf(buf, sizeof buf, "%15s", field);
  }
  out += buf;
}

// Fortran Iw input of columns [a, a+w) of `line`: blanks ignored, an empty
// field reads as 0.  Returns false on a character that is not a digit/sign.
bool get_int(const std::string& line, size_t a, size_t w, long long* v) {
  std::string t;
  for (size_t i = a; i < a + w && i < line.size(); i++)
    if (line[i] != ' ' && line[i] != '\t') t += line[i];
  if (t.empty()) { *v = 0; return true; }
  char* end = nullptr;
  errno = 0;
  *v = std::strtoll(t.c_str(), &end, 10);
  return errno == 0 && end && *end == '\0';
}

// Fortran Ew.d input (d = 8) of columns [a, a+w): blanks ignored; the
// exponent may be written E/D/Q+-n or as a bare signed integer; a field
// without a decimal point has d implied decimal digits.
bool get_e(const std::string& line, size_t a, size_t w, int d, double* v) {
  std::string t;
  for (size_t i = a; i < a + w && i < line.size(); i++)
    if (line[i] != ' ' && line[i] != '\t') t += line[i];
  if (t.empty()) { *v = 0.0; return true; }
  size_t i = 0;
  std::string mant;
  if (t[i] == '+' || t[i] == '-') mant += t[i++];
  bool point = false, digits = false;
  for (; i < t.size(); i++) {
    const char c = t[i];
    if (c >= '0' && c <= '9') { mant += c; digits = true; }
    else if (c == '.' && !point) { mant += c; point = true; }
    else break;
  }
  if (!digits) return false;
  long ex = 0;
  if (i < t.size()) {
    const char c = t[i];
    if (c == 'E' || c == 'e' || c == 'D' || c == 'd' || c == 'Q' || c == 'q') i++;
    if (i >= t.size()) return false;
    char* end = nullptr;
    errno = 0;
    ex = std::strtol(t.c_str() + i, &end, 10);
    if (errno != 0 || !end || *end != '\0' || end == t.c_str() + i) return false;
  }
  if (!point) ex -= d;
  char buf[128];
  std::snprintf(buf, sizeof buf, "%sE%ld", mant.c_str(), ex);
  *v = std::strtod(buf, nullptr);
  return true;
}

bool read_lines(const char* path, std::vector<std::string>& lines) {
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::string cur;
  int c;
  while ((c = std::fgetc(f)) != EOF) {
    if (c == '\n') {
      if (!cur.empty() && cur.back() == '\r') cur.pop_back();
      lines.push_back(cur);
      cur.clear();
    } else {
      cur += (char)c;
    }
  }
  if (!cur.empty()) lines.push_back(cur);
  std::fclose(f);
  return true;
}

}  // namespace

extern "C" {

int neoxc_ufm_read(const char* path, int64_t n, int64_t recl, double* out) {
  const long r = resolve_recl(recl);
  if (!path || n < 0 || (n > 0 && !out) || r < 8)
    return set_last_error(NEOXC_ERR_ARG, "ufm_read: bad arguments (recl %ld)", r);
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return set_last_error(NEOXC_ERR_IO, "ufm_read: cannot open %s", path);
  std::vector<unsigned char> buf((size_t)r);
  int64_t i = 0;
  for (; i < n; i++) {
    // the last record may be short when the writer did not pad it
    const size_t got = std::fread(buf.data(), 1, (size_t)r, f);
    if (got < sizeof(double)) break;
    std::memcpy(&out[i], buf.data(), sizeof(double));
    if (got < (size_t)r) { i++; break; }
  }
  std::fclose(f);
  if (i < n)
    return set_last_error(NEOXC_ERR_IO, "ufm_read: %s holds %lld of %lld records",
                          path, (long long)i, (long long)n);
  return NEOXC_OK;
}

int neoxc_ufm_write(const char* path, const double* v, int64_t n, int64_t recl) {
  const long r = resolve_recl(recl);
  if (!path || n < 0 || (n > 0 && !v) || r < 8)
    return set_last_error(NEOXC_ERR_ARG, "ufm_write: bad arguments (recl %ld)", r);
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return set_last_error(NEOXC_ERR_IO, "ufm_write: cannot open %s", path);
  std::vector<unsigned char> buf((size_t)r, 0);
  bool ok = true;
  for (int64_t i = 0; i < n && ok; i++) {
    std::memcpy(buf.data(), &v[i], sizeof(double));
    ok = std::fwrite(buf.data(), 1, (size_t)r, f) == (size_t)r;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? NEOXC_OK
            : set_last_error(NEOXC_ERR_IO, "ufm_write: short write to %s", path);
}

int neoxc_mo_write(const char* path, int64_t nbf, int64_t nmo, const double* V) {
  if (!path || nbf < 1 || nmo < 0 || (nmo > 0 && !V))
    return set_last_error(NEOXC_ERR_ARG, "mo_write: bad arguments");
  std::string out;
  char lab[32];
  for (int64_t j = 1; j <= nmo; j++) {
    int64_t ic = 0;
    for (int64_t lo = 1; lo <= nbf; lo += 5) {
      ic++;
      const int64_t hi = lo + 4 < nbf ? lo + 4 : nbf;
      std::snprintf(lab, sizeof lab, "%2lld%3lld", (long long)(j % 100),
                    (long long)(ic % 1000));
      out += lab;
      for (int64_t i = lo; i <= hi; i++) put_e15_8(out, V[(i - 1) + nbf * (j - 1)]);
      out += '\n';
    }
  }
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return set_last_error(NEOXC_ERR_IO, "mo_write: cannot open %s", path);
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  return (std::fclose(f) == 0 && ok)
             ? NEOXC_OK
             : set_last_error(NEOXC_ERR_IO, "mo_write: short write to %s", path);
}

int neoxc_mo_read(const char* path, int64_t nbf, int64_t nmo, double* V) {
  if (!path || nbf < 1 || nmo < 0 || (nmo > 0 && !V))
    return set_last_error(NEOXC_ERR_ARG, "mo_read: bad arguments");
  std::vector<std::string> lines;
  if (!read_lines(path, lines))
    return set_last_error(NEOXC_ERR_IO, "mo_read: cannot open %s", path);
  size_t ln = 0;
  for (int64_t j = 1; j <= nmo; j++) {
    int64_t ic = 0;
    for (int64_t lo = 1; lo <= nbf; lo += 5) {
      ic++;
      const int64_t hi = lo + 4 < nbf ? lo + 4 : nbf;
      if (ln >= lines.size())
        return set_last_error(NEOXC_ERR_IO, "mo_read: %s ends at orbital %lld line %lld",
                              path, (long long)j, (long long)ic);
      const std::string& L = lines[ln++];
      long long jj, icc;
      if (!get_int(L, 0, 2, &jj) || !get_int(L, 2, 3, &icc) || jj != j % 100 ||
          icc != ic % 1000)
        return set_last_error(NEOXC_ERR_IO,
                              "mo_read: problem reading orbitals in %s at orbital "
                              "%lld (modulus 100 = %lld), line %lld: read '%.5s'",
                              path, (long long)j, (long long)(j % 100),
                              (long long)ic, L.c_str());
      for (int64_t i = lo; i <= hi; i++) {
        double x;
        if (!get_e(L, 5 + 15 * (size_t)(i - lo), 15, 8, &x))
          return set_last_error(NEOXC_ERR_IO, "mo_read: bad number in %s, orbital %lld "
                                "row %lld", path, (long long)j, (long long)ic);
        V[(i - 1) + nbf * (j - 1)] = x;
      }
    }
  }
  return NEOXC_OK;
}

int neoxc_mo_density(int64_t nbf, int64_t kstart, int64_t klast, double prefac,
                     const double* C, double* D) {
  if (nbf < 1 || !C || !D || kstart < 1 || klast > nbf || klast < kstart - 1)
    return set_last_error(NEOXC_ERR_ARG, "mo_density: bad arguments");
  for (int64_t j = 0; j < nbf; j++)
    for (int64_t i = 0; i < nbf; i++) {
      double acc = 0.0;
      for (int64_t k = kstart - 1; k < klast; k++)
        acc += prefac * C[i + nbf * k] * C[j + nbf * k];
      D[i + nbf * j] = acc;
    }
  return NEOXC_OK;
}

int neoxc_enuc_write(const char* path, double E_nuc) {
  if (!path) return set_last_error(NEOXC_ERR_ARG, "enuc_write: path");
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return set_last_error(NEOXC_ERR_IO, "enuc_write: cannot open %s", path);
  const int w = std::fprintf(f, " %.17G\n", E_nuc);
  return (std::fclose(f) == 0 && w > 0)
             ? NEOXC_OK
             : set_last_error(NEOXC_ERR_IO, "enuc_write: short write to %s", path);
}

int neoxc_enuc_read(const char* path, double* E_nuc) {
  if (!path || !E_nuc) return set_last_error(NEOXC_ERR_ARG, "enuc_read: bad arguments");
  std::vector<std::string> lines;
  if (!read_lines(path, lines))
    return set_last_error(NEOXC_ERR_IO, "enuc_read: cannot open %s", path);
  for (const std::string& L : lines) {
    // list-directed input: the first value, a D exponent allowed
    std::string t;
    size_t i = 0;
    while (i < L.size() && (L[i] == ' ' || L[i] == '\t' || L[i] == ',')) i++;
    for (; i < L.size() && L[i] != ' ' && L[i] != '\t' && L[i] != ',' && L[i] != '/'; i++)
      t += (L[i] == 'D' || L[i] == 'd') ? 'E' : L[i];
    if (t.empty()) continue;
    char* end = nullptr;
    const double v = std::strtod(t.c_str(), &end);
    if (!end || *end != '\0')
      return set_last_error(NEOXC_ERR_IO, "enuc_read: bad value '%s' in %s", t.c_str(), path);
    *E_nuc = v;
    return NEOXC_OK;
  }
  return set_last_error(NEOXC_ERR_IO, "enuc_read: no value in %s", path);
}

}  // extern "C"
