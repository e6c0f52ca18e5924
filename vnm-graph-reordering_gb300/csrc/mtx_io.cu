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
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <tuple>
#include <vector>

#include "../../include/vnm_gb300.h"

namespace {

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
  fclose(f);
  normalise(r, c, v, symmetric, std::min(nz, (int)r.size()));
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
  for (int i = 0; i < nnz; ++i) fprintf(f, "%d %d %.2f\n", row[i] + 1, col[i] + 1, (double)val[i]);
  return fclose(f) == 0 ? VNM_OK : VNM_ERR_IO;
}

// The NM stage writes temp.mtx and the VNM stage reads it: values become the
// float64 of their "%.2f" text.
vnm_status vnm_text_nm_values(int nnz, const float* val, double* out) {
  if (nnz < 0 || (nnz > 0 && (!val || !out))) return VNM_ERR_ARG;
  char b[64];
  for (int i = 0; i < nnz; ++i) {
    snprintf(b, sizeof b, "%.2f", (double)val[i]);
    out[i] = strtod(b, nullptr);
  }
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
  char b[64];
  for (int i = 0; i < nnz; ++i) {
    if (sym != 0 && row[i] < col[i]) continue;  // lower triangle only
    snprintf(b, sizeof b, "%.0e", val[i]);
    r.push_back(row[i]);
    c.push_back(col[i]);
    v.push_back(strtof(b, nullptr));
  }
  normalise(r, c, v, sym == 1, (int)r.size());
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
