// Host-side Matrix Market I/O and the text round trips of the `spmm`
// pipeline, behind the C ABI.
//
// The reference reads files with readMtx (mtx/readMtx.hpp:354-425: banner and
// size line of mtx/mmio.hpp, tuples by fscanf, symmetric banners mirrored,
// repeats removed, sorted by (row, col)), pads the row count to a multiple of
// M (mtx/Mtx.h:106-109), writes "%d %d %.2f" lines (mtx/Mtx.h:412-435), and
// between its stages passes the matrix through temp.mtx, which the Python
// stage rewrites with scipy's mmwrite(precision=1) -- "%.0e" values and, for
// matrices under 100 rows whose values are symmetric, only the lower
// triangle under a "symmetric" banner (reordering.py:179-181).  These
// functions reproduce those effects in memory so the drop-in command needs
// no temporary files.
//
// Speed: the reference parses token by token with fscanf and sorts tuples
// with std::sort on one thread.  Here a regular body (one entry per line)
// is read in one piece and parsed by all host threads with hand-written
// integer and decimal parsers, and sorted by parallel chunk sorts and
// merges.  Every shortcut gives the reference's result bit for bit or is
// not taken: a decimal with at most 2^24 in its significand and a power of
// ten within 10^+-10 is m * 10^e (or m / 10^-e) in one float operation of
// two exact floats, hence correctly rounded like strtof / fscanf("%f");
// other numbers go to strtof; a body that is not one entry per line goes to
// the token-by-token reader; a matrix with repeated (row, col) goes to the
// std::sort path, whose order among equal keys decides which values the
// reference keeps.  VNM_MTX_READER=scalar forces the token-by-token reader
// and the std::sort path (for timing and tests).
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/vnm_gb300.h"

namespace {

int host_threads() {
  const unsigned h = std::thread::hardware_concurrency();
  return h < 1 ? 1 : (h > 64 ? 64 : (int)h);
}

// fn(begin, end, part) over `parts` contiguous ranges of [0, n), in threads
template <class F>
void parallel_ranges(size_t n, int parts, F&& fn) {
  if (parts <= 1 || n < 2) {
    fn((size_t)0, n, 0);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < parts; ++t) {
    const size_t b = n * t / parts, e = n * (t + 1) / parts;
    th.emplace_back([&fn, b, e, t] { fn(b, e, t); });
  }
  for (auto& x : th) x.join();
}

bool scalar_forced() {
  const char* e = getenv("VNM_MTX_READER");
  return e && !strcmp(e, "scalar");
}

typedef std::tuple<int, int, float, int> Tup;

bool tup_less(const Tup& a, const Tup& b) {
  if (std::get<0>(a) == std::get<0>(b)) return std::get<1>(a) < std::get<1>(b);
  return std::get<0>(a) < std::get<0>(b);
}

// sort by (row, col) with std::sort over (row, col, val, index) tuples, the
// order the reference's customSort produces (same library, same comparator)
void sort_coo(std::vector<int>& r, std::vector<int>& c, std::vector<float>& v) {
  const int n = (int)r.size();
  std::vector<Tup> t;
  t.reserve(n);
  for (int i = 0; i < n; ++i) t.emplace_back(r[i], c[i], v[i], i);
  std::sort(t.begin(), t.end(), tup_less);
  std::vector<int> r0 = r, c0 = c;
  std::vector<float> v0 = v;
  for (int i = 0; i < n; ++i) {
    const int k = std::get<3>(t[i]);
    r[i] = r0[k];
    c[i] = c0[k];
    v[i] = v0[k];
  }
}

// mirror (symmetric), sort, drop repeated (row, col): rows/cols compact,
// values keep their sorted positions and are truncated, as the reference's
// removeSelfloop does (mtx/readMtx.hpp:152-219)
void normalise(std::vector<int>& r, std::vector<int>& c, std::vector<float>& v, bool mirror, int nread) {
  if (mirror) {
    for (int i = 0; i < nread; ++i)
      if (c[i] != r[i]) {
        const int rr = r[i], cc = c[i];
        const float vv = v[i];
        r.push_back(cc);
        c.push_back(rr);
        v.push_back(vv);
      }
  }
  sort_coo(r, c, v);
  int k = 0;
  for (int i = 0; i < (int)r.size(); ++i) {
    if (i > 0 && r[i] == r[i - 1] && c[i] == c[i - 1]) continue;
    r[k] = r[i];
    c[k] = c[i];
    ++k;
  }
  r.resize(k);
  c.resize(k);
  v.resize(k);
  sort_coo(r, c, v);
}

// (row, col) key and original index, ordered by key then index
struct KeyIdx {
  uint64_t key;
  uint32_t idx;
  bool operator<(const KeyIdx& o) const { return key < o.key || (key == o.key && idx < o.idx); }
};

// Sort by (row, col) on all host threads: chunk sorts, then rounds of
// pairwise merges.  Returns false (and leaves r, c, v alone) when a (row,
// col) repeats, since then the order std::sort gives among equal keys
// matters.
bool sort_unique_fast(std::vector<int>& r, std::vector<int>& c, std::vector<float>& v) {
  const size_t n = r.size();
  std::vector<KeyIdx> a(n), b(n);
  const int T = n < (1u << 16) ? 1 : host_threads();
  parallel_ranges(n, T, [&](size_t lo, size_t hi, int) {
    for (size_t i = lo; i < hi; ++i) a[i] = {((uint64_t)(uint32_t)r[i] << 32) | (uint32_t)c[i], (uint32_t)i};
    std::sort(a.begin() + lo, a.begin() + hi);
  });
  // merge rounds: runs of width w (chunk boundaries of T parts)
  std::vector<size_t> bnd(T + 1);
  for (int t = 0; t <= T; ++t) bnd[t] = n * t / T;
  while (bnd.size() > 2) {
    std::vector<size_t> nb;
    const int pairs = (int)(bnd.size() - 1) / 2;
    std::vector<std::thread> th;
    for (int p = 0; p < pairs; ++p) {
      const size_t lo = bnd[2 * p], mid = bnd[2 * p + 1], hi = bnd[2 * p + 2];
      th.emplace_back([&a, &b, lo, mid, hi] {
        std::merge(a.begin() + lo, a.begin() + mid, a.begin() + mid, a.begin() + hi, b.begin() + lo);
      });
    }
    for (auto& x : th) x.join();
    for (int p = 0; p < pairs; ++p) nb.push_back(bnd[2 * p]);
    if ((bnd.size() - 1) % 2) {  // an odd run left over: copied as is
      const size_t lo = bnd[bnd.size() - 2], hi = bnd.back();
      std::copy(a.begin() + lo, a.begin() + hi, b.begin() + lo);
      nb.push_back(lo);
    }
    nb.push_back(n);
    a.swap(b);
    bnd.swap(nb);
  }
  for (size_t i = 1; i < n; ++i)
    if (a[i].key == a[i - 1].key) return false;
  std::vector<int> r0(n), c0(n);
  std::vector<float> v0(n);
  parallel_ranges(n, T, [&](size_t lo, size_t hi, int) {
    for (size_t i = lo; i < hi; ++i) {
      const uint32_t k = a[i].idx;
      r0[i] = r[k];
      c0[i] = c[k];
      v0[i] = v[k];
    }
  });
  r.swap(r0);
  c.swap(c0);
  v.swap(v0);
  return true;
}

// normalise() with the fast sort when no (row, col) repeats
void normalise_fast(std::vector<int>& r, std::vector<int>& c, std::vector<float>& v, bool mirror, int nread) {
  if (scalar_forced()) {
    normalise(r, c, v, mirror, nread);
    return;
  }
  if (mirror) {
    for (int i = 0; i < nread; ++i)
      if (c[i] != r[i]) {
        const int rr = r[i], cc = c[i];
        const float vv = v[i];
        r.push_back(cc);
        c.push_back(rr);
        v.push_back(vv);
      }
  }
  if (!sort_unique_fast(r, c, v)) normalise(r, c, v, false, (int)r.size());
}

// ---- body parsers ------------------------------------------------------------
inline bool is_blank(char ch) { return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\v' || ch == '\f'; }
inline bool is_space(char ch) { return is_blank(ch) || ch == '\n'; }
inline bool at_token_end(const char* p, const char* end) { return p == end || is_space(*p); }

// an optionally signed decimal integer of at most 10 digits
bool parse_int(const char*& p, const char* end, int& out) {
  const char* q = p;
  bool neg = false;
  if (q < end && (*q == '+' || *q == '-')) neg = *q++ == '-';
  long long x = 0;
  int nd = 0;
  while (q < end && *q >= '0' && *q <= '9' && nd < 11) {
    x = x * 10 + (*q++ - '0');
    ++nd;
  }
  if (nd == 0 || nd > 10 || !at_token_end(q, end)) return false;
  x = neg ? -x : x;
  if (x < INT32_MIN || x > INT32_MAX) return false;
  out = (int)x;
  p = q;
  return true;
}

const float kPow10[11] = {1e0f, 1e1f, 1e2f, 1e3f, 1e4f, 1e5f, 1e6f, 1e7f, 1e8f, 1e9f, 1e10f};

// a number as fscanf("%f") reads it: the exact shortcut when it applies,
// else strtof on the token (the buffer is NUL-terminated)
bool parse_float(const char*& p, const char* end, float& out) {
  const char* s = p;
  const char* q = p;
  bool neg = false;
  if (q < end && (*q == '+' || *q == '-')) neg = *q++ == '-';
  uint64_t m = 0;
  int nd = 0, e10 = 0;
  bool any = false, exact = true;
  while (q < end && *q >= '0' && *q <= '9') {
    const int d = *q++ - '0';
    any = true;
    if (m == 0 && d == 0) continue;
    if (nd < 19) {
      m = m * 10 + d;
      ++nd;
    } else {
      exact = false;
    }
  }
  if (q < end && *q == '.') {
    ++q;
    while (q < end && *q >= '0' && *q <= '9') {
      const int d = *q++ - '0';
      any = true;
      if (m == 0 && d == 0) {
        --e10;
        continue;
      }
      if (nd < 19) {
        m = m * 10 + d;
        ++nd;
        --e10;
      } else {
        exact = false;
      }
    }
  }
  if (any && q < end && (*q == 'e' || *q == 'E')) {
    const char* t = q + 1;
    bool eneg = false;
    if (t < end && (*t == '+' || *t == '-')) eneg = *t++ == '-';
    int ex = 0, ed = 0;
    while (t < end && *t >= '0' && *t <= '9') {
      if (ex < 100000) ex = ex * 10 + (*t - '0');
      ++t;
      ++ed;
    }
    if (ed > 0) {
      e10 += eneg ? -ex : ex;
      q = t;
    }
  }
  if (any && exact && at_token_end(q, end) && (m == 0 || (m <= (1ull << 24) && e10 >= -10 && e10 <= 10))) {
    float f = (float)m;
    if (m != 0) {
      if (e10 > 0) f *= kPow10[e10];
      else if (e10 < 0) f /= kPow10[-e10];
    }
    out = neg ? -f : f;
    p = q;
    return true;
  }
  char* t = nullptr;
  const float f = strtof(s, &t);
  if (t == s || !at_token_end(t, end)) return false;
  out = f;
  p = t;
  return true;
}

// Entries of a body that holds one entry per line (blank lines allowed):
// false on anything else, which the token-by-token reader then handles.
struct BodyPart {
  std::vector<int> r, c;
  std::vector<float> v;
  bool ok = true;
};

void parse_lines(const char* p, const char* end, int kind, BodyPart& out) {
  while (true) {
    while (p < end && is_space(*p)) ++p;
    if (p >= end) return;
    int a, b;
    float x = 1.0f;
    if (!parse_int(p, end, a)) break;
    while (p < end && is_blank(*p)) ++p;
    if (!parse_int(p, end, b)) break;
    while (p < end && is_blank(*p)) ++p;
    if (kind == 0) {
      if (!parse_float(p, end, x)) break;
    } else if (kind == 1) {
      int y;
      if (!parse_int(p, end, y)) break;
      x = (float)y;
    }
    while (p < end && is_blank(*p)) ++p;
    if (p < end && *p != '\n') break;
    out.r.push_back(a);
    out.c.push_back(b);
    out.v.push_back(x);
  }
  out.ok = false;
}

// The whole body of `f` (from its current position) parsed on all host
// threads; false when it is not one entry per line.
bool read_body_fast(FILE* f, int kind, std::vector<int>& r, std::vector<int>& c, std::vector<float>& v) {
  const long start = ftell(f);
  if (start < 0 || fseek(f, 0, SEEK_END) != 0) return false;
  const long stop = ftell(f);
  if (stop < start || fseek(f, start, SEEK_SET) != 0) return false;
  std::string buf((size_t)(stop - start) + 1, '\0');
  const size_t got = fread(&buf[0], 1, (size_t)(stop - start), f);
  buf.resize(got + 1);
  buf[got] = '\0';
  const char* base = buf.data();
  const size_t n = got;
  const int T = n < (1u << 20) ? 1 : host_threads();
  std::vector<size_t> cut(T + 1);
  cut[0] = 0;
  cut[T] = n;
  for (int t = 1; t < T; ++t) {  // chunk starts at line starts
    size_t x = n * t / T;
    while (x < n && base[x - 1] != '\n') ++x;
    cut[t] = std::max(x, cut[t - 1]);
  }
  std::vector<BodyPart> parts(T);
  parallel_ranges((size_t)T, T, [&](size_t lo, size_t hi, int) {
    for (size_t t = lo; t < hi; ++t) {
      parts[t].r.reserve((cut[t + 1] - cut[t]) / 8 + 1);
      parts[t].c.reserve((cut[t + 1] - cut[t]) / 8 + 1);
      parts[t].v.reserve((cut[t + 1] - cut[t]) / 8 + 1);
      parse_lines(base + cut[t], base + cut[t + 1], kind, parts[t]);
    }
  });
  size_t total = 0;
  for (auto& q : parts) {
    if (!q.ok) return false;
    total += q.r.size();
  }
  r.clear();
  c.clear();
  v.clear();
  r.reserve(total);
  c.reserve(total);
  v.reserve(total);
  for (auto& q : parts) {
    r.insert(r.end(), q.r.begin(), q.r.end());
    c.insert(c.end(), q.c.begin(), q.c.end());
    v.insert(v.end(), q.v.begin(), q.v.end());
  }
  return true;
}

template <class T>
T* copy_out(const std::vector<T>& x) {
  T* p = (T*)malloc(sizeof(T) * (x.empty() ? 1 : x.size()));
  if (p && !x.empty()) memcpy(p, x.data(), sizeof(T) * x.size());
  return p;
}

}  // namespace

extern "C" {

vnm_status vnm_mtx_read(const char* path, int aligned, int* nrows, int* ncols, int* nnz, int** row, int** col,
                        float** val) {
  if (!path || !nrows || !ncols || !nnz || !row || !col || !val) return VNM_ERR_ARG;
  FILE* f = fopen(path, "r");
  if (!f) return VNM_ERR_IO;
  char line[1025], banner[64], mtx[64], crd[64], dtype[64], storage[64];
  if (!fgets(line, sizeof line, f) ||
      sscanf(line, "%63s %63s %63s %63s %63s", banner, mtx, crd, dtype, storage) != 5) {
    fclose(f);
    return VNM_ERR_FORMAT;
  }
  for (char* p : {mtx, crd, dtype, storage})
    for (; *p; ++p) *p = (char)tolower((unsigned char)*p);
  int kind = -1;  // 0 real, 1 integer, 2 pattern
  if (!strcmp(dtype, "real")) kind = 0;
  else if (!strcmp(dtype, "integer")) kind = 1;
  else if (!strcmp(dtype, "pattern")) kind = 2;
  const bool known_storage = !strcmp(storage, "general") || !strcmp(storage, "symmetric") ||
                             !strcmp(storage, "hermitian") || !strcmp(storage, "skew-symmetric");
  if (strncmp(banner, "%%MatrixMarket", 14) || strcmp(mtx, "matrix") || strcmp(crd, "coordinate") || kind < 0 ||
      !known_storage) {
    fclose(f);
    return VNM_ERR_FORMAT;
  }
  const bool symmetric = !strcmp(storage, "symmetric");
  int nr = 0, nc = 0, nz = 0;
  do {
    if (!fgets(line, sizeof line, f)) {
      fclose(f);
      return VNM_ERR_FORMAT;
    }
  } while (line[0] == '%');
  if (sscanf(line, "%d %d %d", &nr, &nc, &nz) != 3) {
    int got;
    do {
      got = fscanf(f, "%d %d %d", &nr, &nc, &nz);
      if (got == EOF) {
        fclose(f);
        return VNM_ERR_FORMAT;
      }
    } while (got != 3);
  }
  if (nr < 0 || nc < 0 || nz < 0) {
    fclose(f);
    return VNM_ERR_FORMAT;
  }
  std::vector<int> r, c;
  std::vector<float> v;
  const long body = ftell(f);
  bool fast = !scalar_forced() && body >= 0 && read_body_fast(f, kind, r, c, v);
  if (fast) {
    // the first nz entries, as the token loop below would read them
    if ((long long)r.size() > (long long)nz) {
      r.resize(nz);
      c.resize(nz);
      v.resize(nz);
    }
    bool bad = false;
    parallel_ranges(r.size(), r.size() < (1u << 16) ? 1 : host_threads(), [&](size_t lo, size_t hi, int) {
      bool b = false;
      for (size_t i = lo; i < hi; ++i) {
        if (r[i] < 1 || c[i] < 1 || r[i] > nr || c[i] > nc) b = true;
        r[i] -= 1;
        c[i] -= 1;
      }
      if (b) bad = true;
    });
    if (bad) {
      fclose(f);
      return VNM_ERR_FORMAT;
    }
  } else {
    if (body < 0 || fseek(f, body, SEEK_SET) != 0) {
      fclose(f);
      return VNM_ERR_IO;
    }
    r.clear();
    c.clear();
    v.clear();
    r.reserve(nz);
    c.reserve(nz);
    v.reserve(nz);
    for (int i = 0; i < nz; ++i) {
      int a, b;
      if (fscanf(f, "%d", &a) == EOF) break;
      if (fscanf(f, "%d", &b) != 1) break;
      float x = 1.0f;
      if (kind == 0) {
        float y = 0.f;
        if (fscanf(f, "%f", &y) == 1) x = y;
      } else if (kind == 1) {
        int y = 0;
        if (fscanf(f, "%d", &y) == 1) x = (float)y;
      }
      if (a < 1 || b < 1 || a > nr || b > nc) {
        fclose(f);
        return VNM_ERR_FORMAT;
      }
      r.push_back(a - 1);
      c.push_back(b - 1);
      v.push_back(x);
    }
  }
  fclose(f);
  normalise_fast(r, c, v, symmetric, std::min(nz, (int)r.size()));
  if (aligned > 0 && nr % aligned != 0) {
    nr = (nr + aligned - 1) / aligned * aligned;
    nc = (nc + aligned - 1) / aligned * aligned;
  }
  *nrows = nr;
  *ncols = nc;
  *nnz = (int)r.size();
  *row = copy_out(r);
  *col = copy_out(c);
  *val = copy_out(v);
  return (*row && *col && *val) ? VNM_OK : VNM_ERR_NOMEM;
}

void vnm_host_free(void* p) { free(p); }

vnm_status vnm_mtx_write(const char* path, int nrows, int ncols, int nnz, const int* row, const int* col,
                         const float* val) {
  if (!path || nnz < 0 || (nnz > 0 && (!row || !col || !val))) return VNM_ERR_ARG;
  FILE* f = fopen(path, "w");
  if (!f) return VNM_ERR_IO;
  fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n%d %d %d\n", nrows, ncols, nnz);
  // the lines are formatted on all host threads (same snprintf), written in order
  const int T = nnz < (1 << 16) ? 1 : host_threads();
  std::vector<std::string> out(T);
  parallel_ranges((size_t)nnz, T, [&](size_t lo, size_t hi, int t) {
    std::string& o = out[t];
    o.reserve((hi - lo) * 24);
    char b[96];
    for (size_t i = lo; i < hi; ++i) {
      const int k = snprintf(b, sizeof b, "%d %d %.2f\n", row[i] + 1, col[i] + 1, (double)val[i]);
      o.append(b, (size_t)k);
    }
  });
  bool ok = true;
  for (auto& o : out) ok = ok && fwrite(o.data(), 1, o.size(), f) == o.size();
  return (fclose(f) == 0 && ok) ? VNM_OK : VNM_ERR_IO;
}

// The NM stage writes temp.mtx and the VNM stage reads it: values become the
// float64 of their "%.2f" text.
vnm_status vnm_text_nm_values(int nnz, const float* val, double* out) {
  if (nnz < 0 || (nnz > 0 && (!val || !out))) return VNM_ERR_ARG;
  parallel_ranges((size_t)nnz, nnz < (1 << 16) ? 1 : host_threads(), [&](size_t lo, size_t hi, int) {
    char b[64];
    for (size_t i = lo; i < hi; ++i) {
      snprintf(b, sizeof b, "%.2f", (double)val[i]);
      out[i] = strtod(b, nullptr);
    }
  });
  return VNM_OK;
}

// The VNM stage rewrites temp.mtx (scipy mmwrite, precision=1) and the NM
// stage reads it back with readMtx.  In: the VNM stage's matrix (n x n,
// entries in its order, float64 values).  Out: the NM reader's COO (sorted,
// mirrored when the writer chose "symmetric"), malloc'ed.  scipy picks
// "symmetric" only when n < 100 and the values are symmetric; a
// skew-symmetric choice is written but not mirrored back by the reader.
vnm_status vnm_text_vnm_roundtrip(int n, int nnz, const int* row, const int* col, const double* val, int aligned,
                                  int* out_nrows, int* out_nnz, int** out_row, int** out_col, float** out_val) {
  if (n < 0 || nnz < 0 || !out_nrows || !out_nnz || !out_row || !out_col || !out_val) return VNM_ERR_ARG;
  int sym = 0;  // 0 general, 1 symmetric, 2 skew-symmetric
  if (n < 100) {
    long up = 0, lo = 0;
    for (int i = 0; i < nnz; ++i) {
      if (val[i] == 0.0) continue;
      if (row[i] < col[i]) ++up;
      else if (row[i] > col[i]) ++lo;
    }
    if (up == lo) {
      std::vector<std::tuple<int, int, double>> e;
      e.reserve(nnz);
      for (int i = 0; i < nnz; ++i) e.emplace_back(row[i], col[i], val[i]);
      std::sort(e.begin(), e.end(), [](const std::tuple<int, int, double>& a, const std::tuple<int, int, double>& b) {
        return std::make_pair(std::get<0>(a), std::get<1>(a)) < std::make_pair(std::get<0>(b), std::get<1>(b));
      });
      auto find = [&](int i, int j) -> double {
        size_t lo2 = 0, hi2 = e.size();
        while (lo2 < hi2) {
          const size_t mid = (lo2 + hi2) / 2;
          if (std::make_pair(std::get<0>(e[mid]), std::get<1>(e[mid])) < std::make_pair(i, j)) lo2 = mid + 1;
          else hi2 = mid;
        }
        if (lo2 < e.size() && std::get<0>(e[lo2]) == i && std::get<1>(e[lo2]) == j) return std::get<2>(e[lo2]);
        return 0.0;
      };
      bool issymm = true, isskew = true;
      for (auto& t : e) {
        const int i = std::get<0>(t), j = std::get<1>(t);
        if (i < j) continue;
        const double aij = std::get<2>(t), aji = i == j ? aij : find(j, i);
        if (isskew && i == j && aij != 0) {
          isskew = false;
        } else {
          if (issymm && aij != aji) issymm = false;
          if (isskew && aij != -aji) isskew = false;
        }
        if (!(issymm || isskew)) break;
      }
      sym = issymm ? 1 : (isskew ? 2 : 0);
    }
  }
  std::vector<int> r, c;
  std::vector<float> v;
  std::vector<float> tv(nnz > 0 ? nnz : 1);
  parallel_ranges((size_t)nnz, nnz < (1 << 16) ? 1 : host_threads(), [&](size_t lo, size_t hi, int) {
    char b[64];
    for (size_t i = lo; i < hi; ++i) {
      snprintf(b, sizeof b, "%.0e", val[i]);
      tv[i] = strtof(b, nullptr);
    }
  });
  for (int i = 0; i < nnz; ++i) {
    if (sym != 0 && row[i] < col[i]) continue;  // lower triangle only
    r.push_back(row[i]);
    c.push_back(col[i]);
    v.push_back(tv[i]);
  }
  normalise_fast(r, c, v, sym == 1, (int)r.size());
  int nr = n;
  if (aligned > 0 && nr % aligned != 0) nr = (nr + aligned - 1) / aligned * aligned;
  *out_nrows = nr;
  *out_nnz = (int)r.size();
  *out_row = copy_out(r);
  *out_col = copy_out(c);
  *out_val = copy_out(v);
  return (*out_row && *out_col && *out_val) ? VNM_OK : VNM_ERR_NOMEM;
}

}  // extern "C"
