// mm.cpp -- Matrix Market reader: mm_matrix (E/MATRIX_MARKET/mm_module.f90:
// 48-154) with the conversions mm_dense (:156-318), mm_crs (:320-540) and
// mm_coo (:542-738), for one process (all rows are local).  The file format
// is the NIST Matrix Market exchange format that the reference reads through
// the mminfo/mmread routines: a banner line, '%' comment lines, a size line,
// then coordinate entries "i j [re [im]]" or array values in column order
// (symmetric / skew / Hermitian arrays store the lower triangle).
//
// Reference behaviours kept: complex entries pass through single precision
// (mmread stores them in default-kind COMPLEX); integer entries become real
// values (crs_format stores ival into rval); symmetric, skew-symmetric and
// Hermitian coordinate files are expanded entry by entry, each mirrored entry
// right after its original (so rows keep the file's order).  Pattern files
// get unit values.  Host code only: idrs_mm_read makes no CUDA call.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/idrs_gb300.h"

namespace idrs {
void set_error(const std::string& msg);
}

namespace {

enum { REP_COORD = 0, REP_ARRAY = 1 };
enum { F_REAL = 0, F_COMPLEX = 1, F_INTEGER = 2, F_PATTERN = 3 };
enum { S_GENERAL = 0, S_SYMMETRIC = 1, S_SKEW = 2, S_HERMITIAN = 3 };

struct MMFile {
  int rep = REP_COORD, field = F_REAL, symm = S_GENERAL;
  int rows = 0, cols = 0;
  long entries = 0;                 // stored entries (coordinate) or values (array)
  std::vector<int> i, j;            // 1-based (coordinate)
  std::vector<double> re, im;       // values (im only for complex)
};

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// Fortran list-directed input also accepts D exponents
double to_double(std::string tok) {
  for (char& c : tok)
    if (c == 'd' || c == 'D') c = 'e';
  char* end = nullptr;
  double v = std::strtod(tok.c_str(), &end);
  if (end == tok.c_str()) throw std::runtime_error("mm: bad number '" + tok + "'");
  return v;
}

bool next_data_line(std::istream& in, std::string& line) {
  while (std::getline(in, line)) {
    size_t p = line.find_first_not_of(" \t\r");
    if (p == std::string::npos) continue;
    if (line[p] == '%') continue;
    return true;
  }
  return false;
}

MMFile parse(const char* path) {
  std::ifstream in(path);
  if (!in) throw std::runtime_error(std::string("Error while opening matrix-market file ") + path);
  MMFile f;
  std::string line;
  if (!std::getline(in, line)) throw std::runtime_error("mm: empty file");
  std::istringstream banner(line);
  std::string tag, object, rep, field, symm;
  banner >> tag >> object >> rep >> field >> symm;
  tag = lower(tag); object = lower(object); rep = lower(rep); field = lower(field); symm = lower(symm);
  if (tag != "%%matrixmarket") throw std::runtime_error("mm: missing %%MatrixMarket banner");
  if (object != "matrix") throw std::runtime_error("mm: only matrix objects are supported");
  if (rep == "coordinate") f.rep = REP_COORD;
  else if (rep == "array") f.rep = REP_ARRAY;
  else throw std::runtime_error("mm: unknown representation " + rep);
  if (field == "real" || field == "double") f.field = F_REAL;
  else if (field == "complex") f.field = F_COMPLEX;
  else if (field == "integer") f.field = F_INTEGER;
  else if (field == "pattern") f.field = F_PATTERN;
  else throw std::runtime_error("mm: unknown field " + field);
  if (symm == "general") f.symm = S_GENERAL;
  else if (symm == "symmetric") f.symm = S_SYMMETRIC;
  else if (symm == "skew-symmetric") f.symm = S_SKEW;
  else if (symm == "hermitian") f.symm = S_HERMITIAN;
  else throw std::runtime_error("mm: unknown symmetry " + symm);
  if (f.rep == REP_ARRAY && f.field == F_PATTERN) throw std::runtime_error("mm: pattern arrays are invalid");
  if (f.symm == S_HERMITIAN && f.field != F_COMPLEX) throw std::runtime_error("mm: Hermitian needs complex");
  if (!next_data_line(in, line)) throw std::runtime_error("mm: missing size line");
  std::istringstream sz(line);
  long rows = -1, cols = -1, nnz = -1;
  sz >> rows >> cols;
  if (f.rep == REP_COORD) sz >> nnz;
  if (rows < 0 || cols < 0 || (f.rep == REP_COORD && nnz < 0) || rows > 2147483647L || cols > 2147483647L)
    throw std::runtime_error("mm: bad size line");
  f.rows = (int)rows;
  f.cols = (int)cols;
  if (f.rep == REP_ARRAY) {
    if (f.symm == S_GENERAL) nnz = rows * cols;
    else if (f.symm == S_SKEW) nnz = rows * (rows - 1) / 2;
    else nnz = rows * (rows + 1) / 2;
    if (f.symm != S_GENERAL && rows != cols) throw std::runtime_error("mm: symmetric array must be square");
  }
  f.entries = nnz;
  if (f.rep == REP_COORD) { f.i.resize(nnz); f.j.resize(nnz); }
  if (f.field != F_PATTERN) f.re.resize(nnz);
  if (f.field == F_COMPLEX) f.im.resize(nnz);
  // values may be spread over lines arbitrarily (list-directed input)
  std::string tok;
  auto need = [&](std::string& t) {
    if (!(in >> t)) throw std::runtime_error("mm: file ends before all entries were read");
  };
  for (long k = 0; k < nnz; ++k) {
    if (f.rep == REP_COORD) {
      need(tok); long a = std::strtol(tok.c_str(), nullptr, 10);
      need(tok); long b = std::strtol(tok.c_str(), nullptr, 10);
      if (a < 1 || a > rows || b < 1 || b > cols) throw std::runtime_error("mm: entry index out of range");
      f.i[k] = (int)a;
      f.j[k] = (int)b;
    }
    if (f.field == F_PATTERN) continue;
    need(tok);
    double re = to_double(tok);
    if (f.field == F_COMPLEX) {
      need(tok);
      double im = to_double(tok);
      f.re[k] = (double)(float)re;  // default-kind COMPLEX in mmread
      f.im[k] = (double)(float)im;
    } else {
      f.re[k] = re;
    }
  }
  return f;
}

bool mirrored(const MMFile& f) { return f.symm != S_GENERAL; }

// value of entry k, and of its mirror (skew: negated, Hermitian: conjugated)
void value(const MMFile& f, long k, bool mirror, double& re, double& im) {
  re = f.field == F_PATTERN ? 1.0 : f.re[k];
  im = f.field == F_COMPLEX ? f.im[k] : 0.0;
  if (!mirror) return;
  if (f.symm == S_SKEW) { re = -re; im = -im; }
  if (f.symm == S_HERMITIAN) im = -im;
}

struct Out {
  int rep = 0, field = 0, nrows = 0, ncols = 0;
  long nnz = 0;
  std::vector<int> ptr, ind;  // crs: row_ptr / col_ind, coo: indx / jndx (1-based)
  std::vector<double> vals;   // real, or interleaved complex
};

Out convert(const MMFile& f, bool crs) {
  Out o;
  o.rep = f.rep;
  o.field = f.field;
  o.nrows = f.rows;
  o.ncols = f.cols;
  const bool cplx = f.field == F_COMPLEX;
  const int vw = cplx ? 2 : 1;
  if (f.rep == REP_ARRAY) {  // mm_dense: column-major nrows x ncols
    o.nnz = (long)f.rows * f.cols;
    o.vals.assign((size_t)o.nnz * vw, 0.0);
    auto put = [&](long r, long c, double re, double im) {
      o.vals[(size_t)(r + (long)f.rows * c) * vw] = re;
      if (cplx) o.vals[(size_t)(r + (long)f.rows * c) * vw + 1] = im;
    };
    long k = 0;
    for (long c = 0; c < f.cols; ++c) {
      long r0 = f.symm == S_GENERAL ? 0 : (f.symm == S_SKEW ? c + 1 : c);
      for (long r = r0; r < f.rows; ++r, ++k) {
        double re, im;
        value(f, k, false, re, im);
        put(r, c, re, im);
        if (f.symm != S_GENERAL) {  // the mirror is written second (also on the diagonal)
          value(f, k, true, re, im);
          put(c, r, re, im);
        }
      }
    }
    return o;
  }
  // coordinate: expanded entry list, each mirror right after its entry
  long total = 0;
  for (long k = 0; k < f.entries; ++k) total += (mirrored(f) && f.i[k] != f.j[k]) ? 2 : 1;
  o.nnz = total;
  o.vals.resize((size_t)total * vw);
  if (crs) {
    std::vector<long> cnt(f.rows + 1, 0);
    for (long k = 0; k < f.entries; ++k) {
      cnt[f.i[k]]++;
      if (mirrored(f) && f.i[k] != f.j[k]) cnt[f.j[k]]++;
    }
    o.ptr.assign(f.rows + 1, 1);
    for (int r = 1; r <= f.rows; ++r) o.ptr[r] = o.ptr[r - 1] + (int)cnt[r];
    o.ind.resize(total);
    std::vector<long> fill(f.rows, 0);
    auto add = [&](int r, int c, double re, double im) {
      long p = o.ptr[r - 1] - 1 + fill[r - 1]++;
      o.ind[p] = c;
      o.vals[(size_t)p * vw] = re;
      if (cplx) o.vals[(size_t)p * vw + 1] = im;
    };
    for (long k = 0; k < f.entries; ++k) {
      double re, im;
      value(f, k, false, re, im);
      add(f.i[k], f.j[k], re, im);
      if (mirrored(f) && f.i[k] != f.j[k]) {
        value(f, k, true, re, im);
        add(f.j[k], f.i[k], re, im);
      }
    }
  } else {
    o.ptr.resize(total);
    o.ind.resize(total);
    long p = 0;
    auto add = [&](int r, int c, double re, double im) {
      o.ptr[p] = r;
      o.ind[p] = c;
      o.vals[(size_t)p * vw] = re;
      if (cplx) o.vals[(size_t)p * vw + 1] = im;
      ++p;
    };
    for (long k = 0; k < f.entries; ++k) {
      double re, im;
      value(f, k, false, re, im);
      add(f.i[k], f.j[k], re, im);
      if (mirrored(f) && f.i[k] != f.j[k]) {
        value(f, k, true, re, im);
        add(f.j[k], f.i[k], re, im);
      }
    }
  }
  return o;
}

bool want_crs(const char* which_format) {
  if (!which_format) return false;  // the reference's default is 'coo'
  std::string w = lower(which_format);
  if (w == "crs") return true;
  if (w == "coo") return false;
  throw std::runtime_error("mm_matrix: which_format must be 'coo' or 'crs'");
}

template <class F>
int mm_guard(F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    idrs::set_error("host allocation failed");
    return IDRS_ERR_ALLOC;
  } catch (const std::exception& e) {
    idrs::set_error(e.what());
    return IDRS_ERR_ARG;
  }
}

}  // namespace

extern "C" {

int idrs_mm_read(const char* mm_file, const char* which_format, int* rep, int* field, int* nrows,
                 int* ncols, long* nnz, int* ptr, int* ind, double* vals) {
  return mm_guard([&] {
    if (!mm_file) throw std::runtime_error("mm_read: no file name");
    const bool crs = want_crs(which_format);
    MMFile f = parse(mm_file);
    Out o = convert(f, crs);
    if (rep) *rep = o.rep;
    if (field) *field = o.field;
    if (nrows) *nrows = o.nrows;
    if (ncols) *ncols = o.ncols;
    if (nnz) *nnz = o.nnz;
    if (ptr && !o.ptr.empty()) std::memcpy(ptr, o.ptr.data(), sizeof(int) * o.ptr.size());
    if (ind && !o.ind.empty()) std::memcpy(ind, o.ind.data(), sizeof(int) * o.ind.size());
    if (vals && !o.vals.empty()) std::memcpy(vals, o.vals.data(), sizeof(double) * o.vals.size());
    return IDRS_OK;
  });
}

int idrs_mm_matrix(const char* mm_file, const char* which_format, idrs_user_matrix* A) {
  int st = mm_guard([&] {
    if (!mm_file || !A) throw std::runtime_error("mm_matrix: bad arguments");
    return IDRS_OK;
  });
  if (st) return st;
  Out o;
  st = mm_guard([&] {
    const bool crs = want_crs(which_format);
    o = convert(parse(mm_file), crs);
    return IDRS_OK;
  });
  if (st) return st;
  const bool cplx = o.field == F_COMPLEX;
  const double* rv = cplx ? nullptr : o.vals.data();
  const double* cv = cplx ? o.vals.data() : nullptr;
  if (o.field == F_PATTERN) rv = nullptr;
  if (o.rep == REP_ARRAY) return idrs_dense_format(o.nrows, o.ncols, rv, cv, A);
  if (which_format && lower(which_format) == "crs")
    return idrs_crs_format(o.nrows, o.ncols, o.ptr.data(), o.ind.data(), rv, cv, A);
  return idrs_coo_format(o.nrows, o.ncols, (int)o.nnz, o.ptr.data(), o.ind.data(), rv, cv, A);
}

}  // extern "C"
