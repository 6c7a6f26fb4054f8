// Host FP64 reference for the error report of the Ozaki path.
//
// An emulated result reports its relative Frobenius error against FP64
// arithmetic on the host over a few sampled result columns (side Left) or
// rows (side Right).  Each reference entry is a compensated dot product
// (Dot2 of Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J.
// Sci. Comput. 26(6), 2005): TwoProduct by one fma, TwoSum by six additions,
// the error terms summed alongside, so the entry is as accurate as if the
// dot product had been computed in twice the working precision and rounded.
// A plain FP64 dot product would carry an error of K * eps * |A||b| itself
// and could not resolve the emulated product's error of ~1e-16.  The file is
// compiled with -ffp-contract=off (the build's host flags) so the error-free
// transformations are not fused away.
//
// op(A) is read in whichever order is contiguous: "dot form" when the
// output entry's row of op(A) is a column of A (y_r = sum_k X[k + r ld] b_k),
// "axpy form" otherwise (y_r = sum_k X[r + k ld] b_k, k outer, one running
// compensated sum per output entry), so A is streamed, never strided.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "api_internal.h"

namespace uvt {

namespace {

struct Acc {
  double p = 0.0, c = 0.0;
  inline void add(double x, double b) {
    const double h = x * b;
    const double r = std::fma(x, b, -h);
    const double t = p + h;
    const double z = t - p;
    const double q = (p - (t - z)) + (h - z);
    p = t;
    c += q + r;
  }
  inline double value() const { return p + c; }
};

struct Job {
  const double *X;
  int64_t ld, len;  // output entries r and dot length k both run over [0, len)
  bool dot_form;    // M(r, k) = X[k + r ld] (true) or X[r + k ld] (false)
  bool k_le_r;      // M(r, k) != 0 only for k <= r (else k >= r)
  bool unit;        // M(r, r) = 1
  double alpha;
  int S;
  const double *b;  // S input vectors, stride len
  double *y;        // S outputs, stride len
};

inline double elem(const Job &j, int64_t r, int64_t k) {
  if (k == r && j.unit) return 1.0;
  return j.dot_form ? j.X[k + r * j.ld] : j.X[r + k * j.ld];
}

// Output entries [r0, r1) of every vector.
void run_rows(const Job &j, int64_t r0, int64_t r1, std::vector<Acc> &acc) {
  const int64_t nr = r1 - r0;
  acc.assign((size_t)nr * j.S, Acc{});
  if (j.dot_form) {
    // One pass over the column; the S sampled vectors are S independent sums.
    for (int64_t r = r0; r < r1; ++r) {
      const int64_t kb = j.k_le_r ? 0 : r, ke = j.k_le_r ? r + 1 : j.len;
      Acc *a = &acc[(size_t)(r - r0) * j.S];
      for (int64_t k = kb; k < ke; ++k) {
        const double x = elem(j, r, k);
        for (int s = 0; s < j.S; ++s) a[s].add(x, j.b[(int64_t)s * j.len + k]);
      }
    }
  } else {
    const int64_t kb = j.k_le_r ? 0 : r0, ke = j.k_le_r ? r1 : j.len;
    for (int64_t k = kb; k < ke; ++k) {
      const int64_t lo = j.k_le_r ? std::max(r0, k) : r0, hi = j.k_le_r ? r1 : std::min(r1, k + 1);
      for (int64_t r = lo; r < hi; ++r) {
        const double x = elem(j, r, k);
        for (int s = 0; s < j.S; ++s) acc[(size_t)(r - r0) * j.S + s].add(x, j.b[(int64_t)s * j.len + k]);
      }
    }
  }
  for (int64_t r = r0; r < r1; ++r)
    for (int s = 0; s < j.S; ++s) j.y[(int64_t)s * j.len + r] = j.alpha * acc[(size_t)(r - r0) * j.S + s].value();
}

void run_job(const Job &j) {
  const int64_t chunk = 64;
  const int64_t nchunks = (j.len + chunk - 1) / chunk;
  std::atomic<int64_t> next{0};
  auto work = [&]() {
    std::vector<Acc> acc;
    for (int64_t c = next++; c < nchunks; c = next++) run_rows(j, c * chunk, std::min(j.len, (c + 1) * chunk), acc);
  };
  const int64_t hw = std::max(1u, std::thread::hardware_concurrency());
  const int nt = (int)std::min<int64_t>(std::min<int64_t>(hw, 64), nchunks);
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) {
    try {
      pool.emplace_back(work);
    } catch (...) {
      break;  // fewer threads; the calling thread still does the rest
    }
  }
  work();
  for (auto &th : pool) th.join();
}

}  // namespace

double host_ref_relerr(const Trmm &t, const double *A, int64_t lda, int S, const double *b, const double *got) {
  const bool left = t.side == CblasLeft;
  const bool lower = (t.uplo == CblasLower) != (t.trans != 0);  // op(A) lower triangular
  Job j;
  j.X = A;
  j.ld = lda;
  j.len = left ? t.m : t.n;
  // Side Left: y_i = sum_k op(A)[i, k] b_k; op(A)[i, k] = A[k + i lda] when transposed.
  // Side Right: y_j = sum_k b_k op(A)[k, j]; op(A)[k, j] = A[k + j lda] when not transposed.
  j.dot_form = left ? t.trans != 0 : t.trans == 0;
  j.k_le_r = left ? lower : !lower;
  j.unit = t.unit != 0;
  j.alpha = t.alpha;
  j.S = S;
  j.b = b;
  std::vector<double> ref((size_t)S * j.len);
  j.y = ref.data();
  run_job(j);
  double num = 0.0, den = 0.0;
  for (size_t i = 0; i < ref.size(); ++i) {
    const double d = got[i] - ref[i];
    num += d * d;
    den += ref[i] * ref[i];
  }
  return den > 0.0 ? std::sqrt(num / den) : std::sqrt(num);
}

}  // namespace uvt
