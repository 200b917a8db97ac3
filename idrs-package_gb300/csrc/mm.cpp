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
#include <algorithm>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

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

bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

// An index token as strtol reads it (0 when it holds no number, so the range
// check rejects it).  std::from_chars is strtol's grammar without the '+' sign.
long tok_long(const char* b, const char* e) {
  if (e - b > 1 && *b == '+' && b[1] != '+' && b[1] != '-') ++b;
  long v = 0;
  const auto r = std::from_chars(b, e, v);
  return r.ec == std::errc() ? v : 0;
}

// A value token as the reference reads it (Fortran list-directed input also
// accepts D exponents).  std::from_chars rounds decimal input exactly like
// strtod; tokens it does not cover (D exponents, hexadecimal, values out of
// the double range) go through strtod itself.  False when there is no number.
bool tok_double(const char* b, const char* e, double& v) {
  bool slow = e - b > 100;
  for (const char* q = b; q < e && !slow; ++q)
    slow = *q == 'd' || *q == 'D' || *q == 'x' || *q == 'X';
  if (!slow) {
    const char* s = (e - b > 1 && *b == '+' && b[1] != '+' && b[1] != '-') ? b + 1 : b;
    const auto r = std::from_chars(s, e, v);
    if (r.ec == std::errc()) return true;
    if (r.ec != std::errc::result_out_of_range) return false;
  }
  std::string tok(b, e);
  for (char& c : tok)
    if (c == 'd' || c == 'D') c = 'e';
  char* end = nullptr;
  v = std::strtod(tok.c_str(), &end);
  return end != tok.c_str();
}

// The whole file, read-only: mapped when the system allows it (no copy; the
// parsing threads fault the pages in), else read into a heap buffer.
class FileView {
 public:
  explicit FileView(const char* path) {
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) throw std::runtime_error(std::string("Error while opening matrix-market file ") + path);
    struct stat st;
    if (::fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
      void* m = ::mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
      if (m != MAP_FAILED) {
        map_ = m;
        size_ = (size_t)st.st_size;
      }
    }
    if (!map_) {  // pipes, special files, or no mapping: read it
      char tmp[1 << 16];
      for (ssize_t got; (got = ::read(fd, tmp, sizeof tmp)) > 0;) heap_.insert(heap_.end(), tmp, tmp + got);
      size_ = heap_.size();
    }
    ::close(fd);
  }
  ~FileView() {
    if (map_) ::munmap(map_, size_);
  }
  FileView(const FileView&) = delete;
  FileView& operator=(const FileView&) = delete;
  const char* data() const { return map_ ? static_cast<const char*>(map_) : heap_.data(); }
  size_t size() const { return size_; }

 private:
  void* map_ = nullptr;
  size_t size_ = 0;
  std::vector<char> heap_;
};

// The data section after the size line is a stream of whitespace-separated
// tokens (values may be spread over lines arbitrarily: list-directed input).
// It is cut into one chunk per host thread at whitespace, each thread counts
// its tokens, a prefix sum gives every chunk its first token number, and the
// threads then parse their tokens into place (token t is field t % per of
// entry t / per).  The first error in token order is reported, as a
// sequential read would.
MMFile parse(const char* path) {
  const FileView file(path);
  const char* p = file.data();
  const char* const end = p + file.size();
  auto getline = [&](std::string& line) -> bool {
    if (p >= end) return false;
    const char* q = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
    if (!q) q = end;
    line.assign(p, q);
    p = q < end ? q + 1 : end;
    return true;
  };
  MMFile f;
  std::string line;
  if (!getline(line)) throw std::runtime_error("mm: empty file");
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
  // size line: the first line that is neither blank nor a '%' comment
  bool have = false;
  while (!have && getline(line)) {
    const size_t q = line.find_first_not_of(" \t\r");
    have = q != std::string::npos && line[q] != '%';
  }
  if (!have) throw std::runtime_error("mm: missing size line");
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

  const bool coord = f.rep == REP_COORD;
  const int nval = f.field == F_PATTERN ? 0 : (f.field == F_COMPLEX ? 2 : 1);
  const int per = (coord ? 2 : 0) + nval;
  const long need = nnz * per;
  const long len = end - p;
  int nth = 1;
  if (len >= (1L << 20)) nth = (int)std::min(64u, std::max(1u, std::thread::hardware_concurrency()));
  std::vector<const char*> cb(nth + 1);
  cb[0] = p;
  cb[nth] = end;
  for (int c = 1; c < nth; ++c) {
    const char* q = std::max(cb[c - 1], p + len * c / nth);
    while (q < end && !is_ws(*q)) ++q;  // chunks end at whitespace: no token is split
    cb[c] = q;
  }
  std::vector<long> first(nth + 1, 0);
  std::vector<long> err_tok(nth, -1);
  std::vector<std::string> err_msg(nth);
  auto run = [&](auto&& body) {
    std::vector<std::thread> th;
    for (int c = 1; c < nth; ++c) th.emplace_back(body, c);
    body(0);
    for (auto& t : th) t.join();
  };
  run([&](int c) {  // tokens per chunk
    long n = 0;
    for (const char *q = cb[c], *e = cb[c + 1]; q < e;) {
      while (q < e && is_ws(*q)) ++q;
      if (q >= e) break;
      ++n;
      while (q < e && !is_ws(*q)) ++q;
    }
    first[c + 1] = n;
  });
  for (int c = 0; c < nth; ++c) first[c + 1] += first[c];
  run([&](int c) {  // parse into place
    long t = first[c];
    for (const char *q = cb[c], *e = cb[c + 1]; q < e && t < need; ++t) {
      while (q < e && is_ws(*q)) ++q;
      if (q >= e) break;
      const char* b = q;
      while (q < e && !is_ws(*q)) ++q;
      const long k = t / per;
      const int fld = (int)(t % per);
      if (coord && fld < 2) {
        const long a = tok_long(b, q);
        if (a < 1 || a > (fld == 0 ? rows : cols)) {
          err_tok[c] = t;
          err_msg[c] = "mm: entry index out of range";
          return;
        }
        (fld == 0 ? f.i : f.j)[k] = (int)a;
        continue;
      }
      double v;
      if (!tok_double(b, q, v)) {
        err_tok[c] = t;
        err_msg[c] = "mm: bad number '" + std::string(b, q) + "'";
        return;
      }
      const int vi = fld - (coord ? 2 : 0);
      if (f.field == F_COMPLEX) (vi == 0 ? f.re : f.im)[k] = (double)(float)v;  // default-kind COMPLEX in mmread
      else f.re[k] = v;
    }
  });
  for (int c = 0; c < nth; ++c)  // chunks are in token order: the first error is the earliest
    if (err_tok[c] >= 0) throw std::runtime_error(err_msg[c]);
  if (first[nth] < need) throw std::runtime_error("mm: file ends before all entries were read");
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
