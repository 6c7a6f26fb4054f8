// C ABI of the Ozaki-style emulated FP64 TRMM (see ozaki.cuh for the method).
#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "api_internal.h"
#include "common.cuh"
#include "ozaki.cuh"

namespace uvt {
namespace {

constexpr int kErrSamples = 8;

// Builds the two residue operands of the canonical GEMM for a normalised TRMM.
void operands(const Trmm &t, const double *dA, int64_t lda, const double *dB, int64_t ldb, OzOperand &L,
              OzOperand &R) {
  const bool lower = (t.uplo == CblasLower) != (t.trans != 0);
  if (t.side == CblasLeft) {
    // Lft = op(A) (m x m), Rgt = B (m x n).
    L = OzOperand{dA, lda, t.m, t.m, t.trans != 0, true, true, lower, t.unit != 0};
    R = OzOperand{dB, ldb, t.n, t.m, true, false, false, false, false};
  } else {
    // Lft = B (m x n), Rgt = op(A) (n x n): Rgt[k, j] = op(A)[k, j].
    L = OzOperand{dB, ldb, t.m, t.n, false, false, false, false, false};
    R = OzOperand{dA, lda, t.n, t.n, t.trans == 0, true, false, lower, t.unit != 0};
  }
}

// Sample positions of the error report: S evenly spaced result columns
// (side Left) or rows (side Right) out of `cnt`.
int64_t sample_index(int S, int s, int64_t cnt) { return S > 1 ? (cnt - 1) * s / (S - 1) : 0; }

// Copies the S sampled vectors of the column-major matrix X (leading
// dimension ld; host memory, or device memory when `device`) into `out`,
// vector after vector.
int gather_samples(uvatrmm_handle_t h, const Trmm &t, int S, const double *X, int64_t ld, bool device,
                   double *out) {
  const bool left = t.side == CblasLeft;
  const int64_t len = left ? t.m : t.n, cnt = left ? t.n : t.m;
  for (int s = 0; s < S; ++s) {
    const int64_t idx = sample_index(S, s, cnt);
    double *o = out + (int64_t)s * len;
    if (device) {
      cudaError_t e = left ? cudaMemcpyAsync(o, X + idx * ld, len * 8, cudaMemcpyDeviceToHost, h->stream)
                           : cudaMemcpy2DAsync(o, 8, X + idx, ld * 8, 8, len, cudaMemcpyDeviceToHost, h->stream);
      if (e != cudaSuccess) return cuda_fail(e, "error-report sample");
    } else if (left) {
      std::memcpy(o, X + idx * ld, (size_t)len * 8);
    } else {
      for (int64_t k = 0; k < len; ++k) o[k] = X[idx + k * ld];
    }
  }
  if (device) {
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "error-report sample");
  }
  return UVATRMM_OK;
}

}  // namespace

int ozaki_device(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n,
                 double alpha, const double *dA, int64_t lda, double *dB, int64_t ldb, int moduli, double *relerr,
                 int *bits_out) {
  if (int bad = check_args(layout, side, uplo, transa, diag, m, n, lda, ldb))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  if (moduli != 0 && (moduli < 2 || moduli > kMaxModuli))
    return fail(UVATRMM_EINVAL, "moduli must be 0 (automatic) or 2.." + std::to_string(kMaxModuli));
  const Trmm t = normalise(layout, side, uplo, transa, diag, m, n, alpha);
  if (relerr) *relerr = 0.0;
  if (t.m == 0 || t.n == 0) return ok();
  if (alpha == 0.0) {
    cudaError_t e = cudaMemset2DAsync(dB, ldb * 8, 0, t.m * 8, t.n, h->stream);
    return e == cudaSuccess ? ok() : cuda_fail(e, "zero fill");
  }
  OzOperand L, R;
  operands(t, dA, lda, dB, ldb, L, R);
  OzPlan plan;
  plan.M = t.m;
  plan.N = t.n;
  plan.K = t.side == CblasLeft ? t.m : t.n;
  plan.n_moduli = moduli ? moduli : ozaki_auto_moduli(plan.K);
  plan.bits = ozaki_bits(plan.n_moduli, plan.K);
  plan.Mp = oz_pad_rows(plan.M);
  plan.Np = oz_pad_cols(plan.N);
  plan.Kp = round_up(plan.K, 64);
  if (bits_out) *bits_out = plan.bits;

  // Residue planes per modulus: (Mp + Np) x Kp bf16; passes of G moduli.
  const int64_t per_mod = (plan.Mp + plan.Np) * plan.Kp * 2;
  int G = (int)std::max<int64_t>(1, std::min<int64_t>(plan.n_moduli, (h->ozaki_scratch_mb << 20) / per_mod));
  const size_t e_bytes = (size_t)round_up((plan.Mp + plan.Np) * (int64_t)sizeof(int), 256);
  int *e = static_cast<int *>(workspace(h, 4, e_bytes + sizeof(OzGroupProb)));
  uint16_t *res =
      static_cast<uint16_t *>(workspace(h, 6, (size_t)plan.n_moduli * plan.Mp * plan.Np * sizeof(uint16_t)));
  uint16_t *planes = static_cast<uint16_t *>(workspace(h, 5, (size_t)G * per_mod));
  if (!e || !res || !planes) return uvatrmm_last_status();
  int *e_row = e, *e_col = e + plan.Mp;

  // Error estimate: keep the sampled inputs (columns of B for side Left,
  // rows for side Right) before B is overwritten.
  const int S = relerr ? (int)std::min<int64_t>(kErrSamples, t.side == CblasLeft ? t.n : t.m) : 0;
  double *samp = nullptr;
  const int64_t len = t.side == CblasLeft ? t.m : t.n;  // entries per sampled column / row
  if (S) {
    samp = static_cast<double *>(workspace(h, 7, (size_t)3 * S * round_up(len, 16) * 8));
    if (!samp) return uvatrmm_last_status();
    const int64_t cnt = t.side == CblasLeft ? t.n : t.m;
    for (int s = 0; s < S; ++s) {
      const int64_t idx = S > 1 ? (cnt - 1) * s / (S - 1) : 0;
      cudaError_t ce = t.side == CblasLeft
                           ? cudaMemcpyAsync(samp + s * round_up(len, 16), dB + idx * ldb, len * 8,
                                             cudaMemcpyDeviceToDevice, h->stream)
                           : cudaMemcpy2DAsync(samp + s, S * 8, dB + idx, ldb * 8, 8, len,
                                               cudaMemcpyDeviceToDevice, h->stream);
      if (ce != cudaSuccess) return cuda_fail(ce, "error-estimate sample");
    }
  }

  h->n_sev = 0;
  auto mark = [&](int kind) {
    if (h->stage_timing && h->n_sev < uvatrmm_handle_st::kStageEvents) {
      h->sev_kind[h->n_sev] = kind;
      cudaEventRecord(h->sev[h->n_sev++], h->stream);
    }
  };
  mark(-1);
  int rc = oz_scales(L, e_row, h->stream);
  if (rc == UVATRMM_OK) rc = oz_scales(R, e_col, h->stream);
  if (rc != UVATRMM_OK) return fail(rc, "Ozaki scaling failed to launch");
  mark(0);
  for (int l0 = 0; l0 < plan.n_moduli; l0 += G) {
    const int l1 = std::min(plan.n_moduli, l0 + G);
    uint16_t *LR = planes, *RR = planes + (int64_t)(l1 - l0) * plan.Mp * plan.Kp;
    rc = oz_residues(L, e_row, plan.bits, l0, l1, plan.Mp, plan.Kp, LR, h->stream);
    if (rc == UVATRMM_OK) rc = oz_residues(R, e_col, plan.bits, l0, l1, plan.Np, plan.Kp, RR, h->stream);
    if (rc != UVATRMM_OK) return fail(rc, "Ozaki residue slicing failed to launch");
    mark(1);
    OzGemmLaunch g;
    g.LR = LR;
    g.RR = RR;
    g.res = res;
    g.Mp = plan.Mp; g.Np = plan.Np; g.Kp = plan.Kp;
    g.M = plan.M; g.N = plan.N; g.K = plan.K;
    g.l0 = l0; g.l1 = l1;
    g.n_moduli = plan.n_moduli;
    g.tri_left = t.side == CblasLeft;
    g.tri_lower = (t.uplo == CblasLower) != (t.trans != 0);
    g.status = h->dctl + 1;
    g.num_sms = h->num_sms;
    g.desc = reinterpret_cast<OzGroupProb *>(reinterpret_cast<char *>(e) + e_bytes);
    g.raster_group = h->oz_raster;
    const char *why = nullptr;
    rc = launch_oz_gemm(g, h->stream, &why);
    if (rc != UVATRMM_OK) return fail(rc, why ? why : "residue GEMM launch failed");
    mark(2);
  }
  rc = oz_reassemble(plan, res, e_row, e_col, t.alpha, dB, ldb, h->stream);
  if (rc != UVATRMM_OK) return fail(rc, "CRT reassembly failed to launch");
  mark(3);

  if (S) {
    // Plain FP64 reference for the sampled columns / rows, then the error.
    const int64_t lp = round_up(len, 16);
    double *ref = samp + (int64_t)S * lp, *got = samp + 2 * (int64_t)S * lp;
    const int64_t cnt = t.side == CblasLeft ? t.n : t.m;
    for (int s = 0; s < S; ++s) {
      const int64_t idx = S > 1 ? (cnt - 1) * s / (S - 1) : 0;
      cudaError_t ce = t.side == CblasLeft
                           ? cudaMemcpyAsync(got + s * lp, dB + idx * ldb, len * 8, cudaMemcpyDeviceToDevice,
                                             h->stream)
                           : cudaMemcpy2DAsync(got + s, S * 8, dB + idx, ldb * 8, 8, len, cudaMemcpyDeviceToDevice,
                                               h->stream);
      if (ce != cudaSuccess) return cuda_fail(ce, "error-estimate sample");
    }
    if (t.side == CblasLeft)
      rc = device_trmm(h, CblasColMajor, CblasLeft, t.uplo, t.trans ? CblasTrans : CblasNoTrans,
                       t.unit ? CblasUnit : CblasNonUnit, t.m, S, t.alpha, dA, lda, samp, lp, ref, lp, false,
                       h->schedule, h->shape);
    else
      rc = device_trmm(h, CblasColMajor, CblasRight, t.uplo, t.trans ? CblasTrans : CblasNoTrans,
                       t.unit ? CblasUnit : CblasNonUnit, S, t.n, t.alpha, dA, lda, samp, S, ref, S, false,
                       h->schedule, h->shape);
    if (rc != UVATRMM_OK) return rc;
    rc = t.side == CblasLeft ? rel_frobenius(h, len, S, got, lp, ref, lp, relerr)
                             : rel_frobenius(h, S, len, got, S, ref, S, relerr);
    if (rc != UVATRMM_OK) return rc;
    rc = collect_status(h);
    if (rc != UVATRMM_OK) return rc;
  }
  return ok();
}

void ozaki_operands(const Trmm &t, const double *dA, int64_t lda, const double *dB, int64_t ldb, OzOperand &L,
                    OzOperand &R) {
  operands(t, dA, lda, dB, ldb, L, R);
}

}  // namespace uvt

using namespace uvt;

extern "C" {

UVATRMM_API int uvatrmm_stage_times(uvatrmm_handle_t h, double *ms4) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  if (!ms4) return fail(UVATRMM_EINVAL, "ms4 is NULL");
  std::lock_guard<std::mutex> g(h->mu);
  for (int k = 0; k < 4; ++k) ms4[k] = 0.0;
  if (h->n_sev < 2) return fail(UVATRMM_EINVAL, "no timed Ozaki call (enable UVATRMM_OPT_STAGE_TIMING)");
  cudaError_t e = cudaEventSynchronize(h->sev[h->n_sev - 1]);
  if (e != cudaSuccess) return cuda_fail(e, "stage timing");
  for (int i = 1; i < h->n_sev; ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->sev[i - 1], h->sev[i]);
    if (h->sev_kind[i] >= 0 && h->sev_kind[i] < 4) ms4[h->sev_kind[i]] += ms;
  }
  return ok();
}

UVATRMM_API int uvatrmm_ozaki_plan(int64_t k, int moduli, int *moduli_out, int *bits_out) {
  if (k < 0 || (moduli != 0 && (moduli < 2 || moduli > kMaxModuli))) return fail(UVATRMM_EINVAL, "invalid arguments");
  const int n = moduli ? moduli : ozaki_auto_moduli(k);
  if (moduli_out) *moduli_out = n;
  if (bits_out) *bits_out = ozaki_bits(n, k);
  return ok();
}

UVATRMM_API int uvatrmm_ozaki_dtrmm_device(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag,
                                          int64_t m, int64_t n, double alpha, const double *dA, int64_t lda,
                                          double *dB, int64_t ldb, int moduli, double *relerr_out, int *bits_out) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  std::lock_guard<std::mutex> g(h->mu);
  if (!relerr_out || !h->oz_err_host)
    return ozaki_device(h, layout, side, uplo, transa, diag, m, n, alpha, dA, lda, dB, ldb, moduli, relerr_out,
                        bits_out);
  // Error against the host FP64 reference: the sampled inputs and op(A) are
  // copied to the host around the call.
  if (int bad = check_args(layout, side, uplo, transa, diag, m, n, lda, ldb))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  const Trmm t = normalise(layout, side, uplo, transa, diag, m, n, alpha);
  // Nothing to compare (empty, alpha = 0) or an invalid slice count: the
  // plain path reports it before anything is copied.
  if (t.m == 0 || t.n == 0 || alpha == 0.0 || (moduli != 0 && (moduli < 2 || moduli > kMaxModuli)))
    return ozaki_device(h, layout, side, uplo, transa, diag, m, n, alpha, dA, lda, dB, ldb, moduli, relerr_out,
                        bits_out);
  *relerr_out = 0.0;
  const bool left = t.side == CblasLeft;
  const int64_t len = left ? t.m : t.n, cnt = left ? t.n : t.m, ka = len;
  const int S = (int)std::min<int64_t>(kErrSamples, cnt);
  std::vector<double> b((size_t)S * len), got((size_t)S * len);
  std::unique_ptr<double[]> A;  // host copy of A (not zero-filled: every entry read is copied in)
  if (S && alpha != 0.0) {
    if (int rc = gather_samples(h, t, S, dB, ldb, true, b.data())) return rc;
    A.reset(new (std::nothrow) double[(size_t)ka * ka]);
    if (!A) return fail(UVATRMM_ENOMEM, "host memory for the error report's copy of A");
    cudaError_t e = cudaMemcpy2DAsync(A.get(), ka * 8, dA, lda * 8, ka * 8, ka, cudaMemcpyDeviceToHost, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "error-report copy of A");
  }
  int rc = ozaki_device(h, layout, side, uplo, transa, diag, m, n, alpha, dA, lda, dB, ldb, moduli, nullptr,
                        bits_out);
  if (rc != UVATRMM_OK || !S || alpha == 0.0) return rc;
  if ((rc = collect_status(h)) != UVATRMM_OK) return rc;
  if ((rc = gather_samples(h, t, S, dB, ldb, true, got.data())) != UVATRMM_OK) return rc;
  *relerr_out = host_ref_relerr(t, A.get(), ka, S, b.data(), got.data());
  return ok();
}

UVATRMM_API int uvatrmm_ozaki_dtrmm(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag,
                                   int64_t m, int64_t n, double alpha, const double *A, int64_t lda, double *B,
                                   int64_t ldb, int moduli, double *relerr_out, int *bits_out) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  std::lock_guard<std::mutex> g(h->mu);
  if (int bad = check_args(layout, side, uplo, transa, diag, m, n, lda, ldb))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  const Trmm t = normalise(layout, side, uplo, transa, diag, m, n, alpha);
  if (t.m == 0 || t.n == 0) return ok();
  const int64_t ka = t.side == CblasLeft ? t.m : t.n;
  const int64_t la = round_up(ka, 16), lb = round_up(t.m, 16);
  double *dA = static_cast<double *>(workspace(h, 0, (size_t)la * ka * 8));
  double *dB = static_cast<double *>(workspace(h, 2, (size_t)lb * t.n * 8));
  if (!dA || !dB) return uvatrmm_last_status();
  cudaError_t e = copy_triangle_h2d(h, dA, la, A, lda, ka, t.uplo == CblasLower);
  if (e == cudaSuccess) e = host_copy2d(h, dB, lb * 8, B, ldb * 8, t.m * 8, t.n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
  // Error report: the sampled inputs are kept before B is overwritten; the
  // reference is computed on the host from the caller's own A and B.
  const bool left = t.side == CblasLeft;
  const int64_t len = left ? t.m : t.n, cnt = left ? t.n : t.m;
  const int S = relerr_out && alpha != 0.0 ? (int)std::min<int64_t>(kErrSamples, cnt) : 0;
  if (relerr_out) *relerr_out = 0.0;
  std::vector<double> bs((size_t)S * len), got((size_t)S * len);
  if (S) gather_samples(h, t, S, B, ldb, false, bs.data());
  int rc = ozaki_device(h, CblasColMajor, t.side, t.uplo, t.trans ? CblasTrans : CblasNoTrans,
                        t.unit ? CblasUnit : CblasNonUnit, t.m, t.n, t.alpha, dA, la, dB, lb, moduli, nullptr,
                        bits_out);
  if (rc != UVATRMM_OK) return rc;
  e = host_copy2d(h, B, ldb * 8, dB, lb * 8, t.m * 8, t.n, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
  rc = collect_status(h);
  if (rc != UVATRMM_OK) return rc;
  if (S) {
    gather_samples(h, t, S, B, ldb, false, got.data());
    *relerr_out = host_ref_relerr(t, A, lda, S, bs.data(), got.data());
  }
  return ok();
}

}  // extern "C"
