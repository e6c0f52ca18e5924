// `spmm` -- drop-in for the reference's command (main.cu:339-352), over the
// C ABI of libvnm_gb300.
//
//   spmm --mtxfile F --outmtxfile O --maxiter R --n 64 --sched S --v V
//        [--N n] [--M m] [--device d] [--compat-files]
//
// Flags as util/argparse.h:27-46 parses them: unknown flags are ignored,
// missing ones default to 0 / "", --n is accepted and unused, --sched is
// accepted and ignored (the schedule is searched over 0-3, main.cu:348).
// N and M, compile-time constants in the reference (mtx/Mtx.h:15-16), are
// run-time flags here with the reference's defaults 2 and 8.
//
// Output: the reordered matrix in O ("%d %d %.2f", mtx/Mtx.h:412-435) and
// one CSV line on stdout with the 16 fields of main.cu:331-335.  The
// reference runs its VNM stage as `python3 reordering.py` on temp.mtx; here
// both stages run on the GPU and the effects of that file round trip (value
// rounding, scipy's symmetric write for small matrices) are applied in
// memory.  --compat-files also writes temp.mtx and output.txt in the
// working directory, as the reference leaves them.
//
// find_best_2toX breaks ties on improve rate by each schedule's measured
// wall time (main.cu:90-99); here they go to the lowest schedule id, so the
// result does not depend on timing.  VNM_SPMM_SCHED=s (0-3) in the
// environment fixes the schedule instead, to reproduce a recorded run of
// the reference that picked s among tied schedules.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "vnm_gb300.h"

extern "C" {
vnm_status vnm_mtx_read(const char* path, int aligned, int* nrows, int* ncols, int* nnz, int** row, int** col,
                        float** val);
vnm_status vnm_mtx_write(const char* path, int nrows, int ncols, int nnz, const int* row, const int* col,
                         const float* val);
void vnm_host_free(void* p);
vnm_status vnm_text_nm_values(int nnz, const float* val, double* out);
vnm_status vnm_text_vnm_roundtrip(int n, int nnz, const int* row, const int* col, const double* val, int aligned,
                                  int* out_nrows, int* out_nnz, int** out_row, int** out_col, float** out_val);
}

namespace {

struct Coo {
  int nrows = 0, ncols = 0;
  std::vector<int> row, col;
  std::vector<float> val;
  int nnz() const { return (int)row.size(); }
};

struct Args {
  std::string mtxfile, outmtxfile;
  int maxiter = 0, n = 0, sched = 0, v = 0;
  int N = 2, M = 8, device = 0;
  bool compat = false;
};

Args parse(int argc, const char** argv) {  // util/argparse.h:6-47
  Args a;
  for (int i = 1; i < argc; ++i) {
    const bool has = i != argc - 1;
    if (!strcmp(argv[i], "--mtxfile") && has) a.mtxfile = argv[i + 1];
    else if (!strcmp(argv[i], "--outmtxfile") && has) a.outmtxfile = argv[i + 1];
    else if (!strcmp(argv[i], "--maxiter") && has) a.maxiter = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "--n") && has) a.n = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "--sched") && has) a.sched = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "--v") && has) a.v = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "--N") && has) a.N = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "--M") && has) a.M = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "--device") && has) a.device = atoi(argv[i + 1]);
    else if (!strcmp(argv[i], "--compat-files")) a.compat = true;
  }
  return a;
}

[[noreturn]] void die(const char* what, vnm_status st) {
  fprintf(stderr, "spmm: %s: %s\n", what, vnm_status_string(st));
  exit(1);
}

vnm_status read_coo(const std::string& path, int aligned, Coo& out) {
  int nr, nc, nz, *r, *c;
  float* v;
  vnm_status st = vnm_mtx_read(path.c_str(), aligned, &nr, &nc, &nz, &r, &c, &v);
  if (st != VNM_OK) return st;
  out.nrows = nr;
  out.ncols = nc;
  out.row.assign(r, r + nz);
  out.col.assign(c, c + nz);
  out.val.assign(v, v + nz);
  vnm_host_free(r);
  vnm_host_free(c);
  vnm_host_free(v);
  return VNM_OK;
}

// run_onepair* of schedule `sched` on A, A relabelled in place
void nm_pass(vnm_ctx* ctx, Coo& A, const Args& a, int sched, int res[5]) {
  std::vector<int> newpos(A.nrows > 0 ? A.nrows : 1);
  vnm_status st = vnm_nm_reorder(ctx, A.nrows, A.nnz(), A.row.data(), A.col.data(), A.val.data(), VNM_MEM_HOST,
                                 a.N, a.M, sched, 10, res, newpos.data());
  if (st != VNM_OK) die("NM reorder", st);
  if (A.nnz() > 0) {
    st = vnm_permute_coo(ctx, A.nrows, A.nnz(), A.row.data(), A.col.data(), VNM_MEM_HOST, newpos.data());
    if (st != VNM_OK) die("permute", st);
  }
}

void eval_vnm(vnm_ctx* ctx, int m, int n, const std::vector<int>& r, const std::vector<int>& c, const Args& a,
              int out2[2]) {
  vnm_status st = vnm_vnm_eval(ctx, m, n, (int)r.size(), r.data(), c.data(), VNM_MEM_HOST, a.M, a.v, out2);
  if (st != VNM_OK) die("VNM eval", st);
}

}  // namespace

int main(int argc, const char** argv) {
  const Args a = parse(argc, argv);
  if (a.M < 2 || a.M > 8 || a.N < 1 || a.N >= a.M || a.v < 1 || a.maxiter < 0) {
    fprintf(stderr, "spmm: need 1 <= N < M <= 8, --v >= 1, --maxiter >= 0\n");
    return 1;
  }
  Coo A0;
  vnm_status st = read_coo(a.mtxfile, a.M, A0);
  if (st == VNM_ERR_IO) {  // mtx/readMtx.hpp:370-373
    printf("File %s not found\n", a.mtxfile.c_str());
    return 1;
  }
  if (st != VNM_OK) die("reading the matrix", st);
  vnm_ctx* ctx = nullptr;
  st = vnm_create(&ctx, a.device);
  if (st != VNM_OK) die("CUDA device", st);

  // 1. find_best_2toX over schedules 0-3 (main.cu:72-114)
  int best = 0, res4[20];
  st = vnm_nm_search(ctx, A0.nrows, A0.nnz(), A0.row.data(), A0.col.data(), A0.val.data(), VNM_MEM_HOST, a.N, a.M,
                     10, &best, res4, nullptr);
  if (st != VNM_OK) die("schedule search", st);
  if (const char* e = getenv("VNM_SPMM_SCHED")) {
    const int s = atoi(e);
    if (s >= 0 && s <= 3) best = s;
  }

  // 2. hybrid_reordering (main.cu:195-337)
  Coo A = A0;
  if (A.nnz() == 0) {  // main.cu:204
    std::cout << std::endl;
    vnm_destroy(ctx);
    return 0;
  }
  int venom0[2];
  {
    // eval_venom reads temp.mtx from the working directory (main.cu:207)
    Coo stale;
    if (read_coo("temp.mtx", 1, stale) == VNM_OK)
      eval_vnm(ctx, stale.nrows, stale.ncols, stale.row, stale.col, a, venom0);
    else
      eval_vnm(ctx, A.nrows, A.ncols, A.row, A.col, a, venom0);
  }
  const auto t0 = std::chrono::steady_clock::now();
  int res_first[5], res[5];
  nm_pass(ctx, A, a, best, res_first);
  memcpy(res, res_first, sizeof res);
  std::vector<double> tval(A.nnz());
  vnm_text_nm_values(A.nnz(), A.val.data(), tval.data());  // temp.mtx as written
  Coo out = A;
  Coo cur = A;
  int nm_round = 0, vnm_round = 0;
  for (int it = 0; it < a.maxiter; ++it) {
    // VNM_reordering: reordering.py on temp.mtx (main.cu:262)
    std::vector<int> r = cur.row, c = cur.col;
    int out5[5];
    st = vnm_vnm_reorder(ctx, cur.nrows, cur.ncols, cur.nnz(), r.data(), c.data(), VNM_MEM_HOST, a.M, a.v, 10, out5,
                         nullptr);
    if (st != VNM_OK) die("VNM reorder", st);
    vnm_round += out5[4];
    int nr, nz, *rr, *cc;
    float* vv;
    st = vnm_text_vnm_roundtrip(cur.nrows, cur.nnz(), r.data(), c.data(), tval.data(), a.M, &nr, &nz, &rr, &cc, &vv);
    if (st != VNM_OK) die("temp.mtx round trip", st);
    Coo B;
    B.nrows = B.ncols = nr;
    B.row.assign(rr, rr + nz);
    B.col.assign(cc, cc + nz);
    B.val.assign(vv, vv + nz);
    vnm_host_free(rr);
    vnm_host_free(cc);
    vnm_host_free(vv);
    nm_pass(ctx, B, a, best, res);  // main.cu:268-303
    nm_round += res[4];
    tval.resize(B.nnz());
    vnm_text_nm_values(B.nnz(), B.val.data(), tval.data());
    cur = B;
    if (it == a.maxiter - 1) out = B;
  }
  const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  int venom1[2];
  eval_vnm(ctx, cur.nrows, cur.ncols, cur.row, cur.col, a, venom1);
  const float improve = (res_first[2] != 0) ? ((res_first[2] - res[3]) * 1.0f / res_first[2]) : 0;
  const float density = A0.nnz() * 1.0f / (int)((unsigned)A0.nrows * (unsigned)A0.nrows);
  std::cout << (float)A0.nrows << ", " << (float)A0.nnz() << ", " << density << ", " << (float)res_first[0] << ", "
            << (float)res[1] << ", " << (float)res_first[2] << ", " << (float)res[3] << ", " << improve << ", "
            << venom0[0] << ", " << venom1[0] << ", " << venom0[1] << ", " << venom1[1] << ", " << nm_round << ", "
            << vnm_round << ", " << nm_round + vnm_round << ", " << (float)ms << std::endl;
  if (!a.outmtxfile.empty()) {
    st = vnm_mtx_write(a.outmtxfile.c_str(), out.nrows, out.ncols, out.nnz(), out.row.data(), out.col.data(),
                       out.val.data());
    if (st != VNM_OK) die("writing the output matrix", st);
  }
  if (a.compat) {
    vnm_mtx_write("temp.mtx", cur.nrows, cur.ncols, cur.nnz(), cur.row.data(), cur.col.data(), cur.val.data());
    FILE* f = fopen("output.txt", "w");
    if (f) {
      fprintf(f, "%d,%d", venom1[0], venom1[1]);
      fclose(f);
    }
  }
  vnm_destroy(ctx);
  return 0;
}
