// Golden-vector harness around the reference's own NM reorder (GPU code).
//
// TEST INFRASTRUCTURE ONLY.  oracle/ref_build.py appends this file to the
// reference headers mtx/Mtx.h and reorder/reorder.h (with the N and M that
// mtx/Mtx.h:15-16 fixes at compile time) and builds it with nvcc into
// oracle/_ref/.  It mirrors graph_NM_reordering (main.cu:13-70): read the
// matrix with Mtx<float>(file, M), build reorderUtil<float>(mat, 10), run one
// schedule, then print the result vector and the final COO.
//
// usage: ref_nm <in.mtx> <sched 0..3> <out.txt> [verbose]
// With a fourth argument the reference's own verbose/stepmsg printing of
// run_onepair* is switched on (its per-round lists, swap lists and swaps).
// out.txt: "nrows nnz r0 r1 r2 r3 r4" then nnz lines "row col" (0-based, in
// the COO order that Mtx::write_to_file would print).

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

int main(int argc, char** argv) {
  if (argc != 4 && argc != 5) {
    fprintf(stderr, "usage: %s <in.mtx> <sched> <out.txt> [verbose]\n", argv[0]);
    return 2;
  }
  std::string path = argv[1];
  int sched = atoi(argv[2]);
  bool verbose = argc == 5;
  {  // report whether the scorer can launch with the reference's 1024 threads
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, GetSegSwapScore) == cudaSuccess)
      fprintf(stderr, "GetSegSwapScore: %d registers, max %d threads per block\n", fa.numRegs,
              fa.maxThreadsPerBlock);
  }
  Mtx<float>* spmat = new Mtx<float>(path, M);
  reorderUtil<float>* rutil = new reorderUtil<float>(spmat, 10);
  std::vector<int> res;
  switch (sched) {
    case 0: res = rutil->run_onepair(verbose, verbose); break;
    case 1: res = rutil->run_onepair_double(verbose, verbose); break;
    case 2: res = rutil->run_onepair_reverse(verbose, verbose); break;
    case 3: res = rutil->run_onepair_reverse_double(verbose, verbose); break;
    default: fprintf(stderr, "bad schedule\n"); return 2;
  }
  cudaError_t err = cudaDeviceSynchronize();
  if (err != cudaSuccess) {
    fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(err));
    return 3;
  }
  spmat->get_coo_host();
  FILE* f = fopen(argv[3], "w");
  if (!f) return 4;
  fprintf(f, "%d %d %d %d %d %d %d\n", spmat->nrows, spmat->nnz, res[0], res[1], res[2], res[3], res[4]);
  for (int i = 0; i < spmat->nnz; ++i) fprintf(f, "%d %d\n", spmat->coo_rowind_h[i], spmat->coo_colind_h[i]);
  fclose(f);
  return 0;
}
