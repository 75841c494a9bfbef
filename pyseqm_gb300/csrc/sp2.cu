// SP2 density purification, plain FP64 (SP2.py:9-85 restated per molecule).
//
// X0 = (hN I - F)/(hN - h1) with Gershgorin bounds h1, hN; each step forms X^2
// (FP64 symmetric tile product, one grid slice per molecule) and keeps X^2 or
// 2X - X^2, whichever brings the trace closer to nocc; a molecule stops when the
// trace error of the last two steps is below eps.  The branch test's tr X^2 is
// ||X||_F^2 of the symmetric X.  Each molecule runs at its own size (the
// reference zero-pads the batch to its largest basis).
#include <math.h>

#include "common.cuh"
#include "sp2_common.cuh"

using namespace seqm;

extern "C" int seqm_density_sp2(const seqm_batch *bp, const double *F, double *P, double *work, double eps,
                                const uint8_t *active, int32_t *status, int max_iter, void *stream) {
  if (!bp || !work) return SEQM_E_ARG;
  seqm_batch b = *bp;
  if (b.nmol == 0) return SEQM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  eps = eps > 1.0e-3 ? 1.0e-3 : (eps < 1.0e-7 ? 1.0e-7 : eps);  // SP2.py:27-30 (float64)
  int64_t total = 0;
  if (batch_total(b, s, &total) != SEQM_OK) return SEQM_E_CUDA;
  // work (doubles): X [T] | X2 [T] | state [SP2_NS nmol] | row bounds 2 [nmol max_norb] | counter
  double *X = work, *X2 = work + total, *st = work + 2 * total;
  double *rowlo = st + (size_t)SP2_NS * b.nmol;
  double *rowhi = rowlo + (size_t)b.nmol * b.max_norb;
  int *cnt = reinterpret_cast<int *>(rowhi + (size_t)b.nmol * b.max_norb);
  k_sp2_rows<<<rows_grid(b), 256, 0, s>>>(b, F, rowlo, rowhi, active);
  k_sp2_bounds<<<b.nmol, 256, 0, s>>>(b, rowlo, rowhi, st, active);
  k_sp2_scale<double><<<ew_grid(b), EW_THREADS, 0, s>>>(b, F, X, st);
  k_sp2_start<<<(b.nmol + 127) / 128, 128, 0, s>>>(b, st);
  int rc = SEQM_OK;
  if (stream_capturing(s)) {
    // inside a CUDA graph capture: the step loop becomes a WHILE node that the device ends
    if (cudaMemsetAsync(cnt, 0, LC_WORDS * sizeof(int), s) != cudaSuccess) return SEQM_E_CUDA;
    const cudaError_t e = capture_while_loop(s, [&](cudaGraph_t body, cudaGraphConditionalHandle h) {
      cudaGraphNode_t n0, n1, n2, n3;
      cudaError_t r = add_kernel_node(body, &n0, nullptr, 0, k_sym_gemm<double, false>, gemm64_grid(b),
                                      dim3(MW_THREADS), 0, b, (const double *)X, (const double *)X, X2, active,
                                      (const double *)st);
      if (r == cudaSuccess)
        r = add_kernel_node(body, &n1, &n0, 1, k_sp2_step<double>, ew_grid(b), dim3(EW_THREADS), 0, b, X,
                            (const double *)X2, st);
      if (r == cudaSuccess)
        r = add_kernel_node(body, &n2, &n1, 1, k_sp2_check, dim3((b.nmol + 127) / 128), dim3(128), 0, b, st, eps, 0,
                            cnt + LC_RUN);
      if (r == cudaSuccess)
        r = add_kernel_node(body, &n3, &n2, 1, k_sp2_loop_tail, dim3(1), dim3(1), 0, cnt, h, max_iter);
      return r;
    });
    if (e != cudaSuccess) return SEQM_E_CUDA;
  } else
  for (int it = 0; it < max_iter; ++it) {
    if (cudaMemsetAsync(cnt, 0, sizeof(int), s) != cudaSuccess) { rc = SEQM_E_CUDA; break; }
    k_sym_gemm<double><<<gemm64_grid(b), MW_THREADS, 0, s>>>(b, X, X, X2, active, st);
    k_sp2_step<double><<<ew_grid(b), EW_THREADS, 0, s>>>(b, X, X2, st);
    k_sp2_check<<<(b.nmol + 127) / 128, 128, 0, s>>>(b, st, eps, 0, cnt);
    if ((it + 1) % SP2_SYNC_EVERY != 0 && it + 1 < max_iter) continue;  // finished molecules skip the extra steps
    int h = 0;
    if (cudaMemcpyAsync(&h, cnt, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) { rc = SEQM_E_CUDA; break; }
    if (h == 0) break;
  }
  if (rc != SEQM_OK) return rc;
  if (status) k_sp2_status<<<(b.nmol + 127) / 128, 128, 0, s>>>(b.nmol, st, active, status, nullptr);
  k_ew_axpby<<<ew_grid(b), EW_THREADS, 0, s>>>(b, 2.0, X, 0.0, nullptr, P, active);  // P = 2 X
  return launch_check();
}
