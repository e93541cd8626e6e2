/*
 * CPU oracle for the SDGC sparse-DNN recurrence -- TEST INFRASTRUCTURE ONLY.
 *
 * Nothing in the product links or calls this file.  It is loaded by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and
 * only there as the checker or as the timed CPU baseline.
 *
 * What it restates (paths inside IDEA-CUHK/SNICIT):
 *   oracle_infer       the plain recurrence of bf_inference
 *                      (src/SDGC/BF/kernel.hpp:26-89) driven as BF::_infer does
 *                      (src/SDGC/BF/BF.hpp:157-229): every layer, each non-empty
 *                      row r gets Y1[r][c] = min(clamp, max(0, sum_j Y0[r][j]*W[j][c] + b));
 *                      inputs equal to 0 are skipped (kernel.hpp:65-67); a row
 *                      whose outputs are all <= 0 leaves the row list
 *                      (BF.hpp:222-229) and stays zero.  Weights are CSR by input
 *                      row with duplicate entries already summed
 *                      (tsv_string_to_CSR_packed_array, src/SDGC/utility.hpp:85-126).
 *                      precision 64: double accumulation and double activations
 *                      (the FP64 oracle); precision 32: float, products then sums
 *                      in ascending input order (the CPU baseline "port").
 *   oracle_identify    mode 0: category = any activation > 0 (SNICIT recover,
 *                      src/SDGC/SNICIT/kernel.hpp:197-218, and the SDGC category
 *                      definition); mode 1: the reference's identify
 *                      (src/SDGC/utility.hpp:194-212) as compiled: thrust::reduce
 *                      with an int initial value runs sequentially in device code
 *                      (CCCL 3.0 thrust/system/detail/sequential/reduce.h) and
 *                      truncates the running sum to int after every element, so
 *                      a row is 1 iff some single activation is >= 1.
 *   oracle_snicit      the SNICIT residue form in FP64 (paper Eqs. 3-6;
 *                      coarse_cluster, post_minus, recover in
 *                      src/SDGC/SNICIT/kernel.hpp:8-69,104-136,197-218): plain
 *                      layers below the threshold, then every live row becomes
 *                      centroid + residue (nearest centroid by L0 distance, ties
 *                      to the lowest index), centroids update as y' = f(Wc + b),
 *                      residues as d' = f(Wc + b + Wd) - f(Wc + b), and rows are
 *                      recovered as c + d.
 *   oracle_ref_candidates   the reference's centroid pick: the first 32 live
 *                      rows, 16-bin sums read as reduction() indexes them
 *                      (src/SDGC/SNICIT/kernel.hpp:138-153, including the
 *                      overlapping bins for N > 1024), greedy pruning with
 *                      eps = 0.03 (centroid_sel, kernel.hpp:156-194).
 *
 * Parity pins: the golden fixtures under tests/golden/ (outputs of the
 * reference's own bf_inference / snig_inference kernels, compiled from its
 * sources and run on a GB300) are checked against oracle_infer by the CPU
 * tests.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int N, L, precision;
  const int32_t* row_off; /* L * (N + 1), layer-local offsets */
  const int32_t* cols;    /* concatenated, layer base nnz_off[l] */
  const float* vals;
  const int64_t* nnz_off; /* L + 1 */
  const float* bias_vec;  /* L * N or NULL */
  float bias, clampv;
  const float* Y0;
  int64_t r0, r1;
  double* outY64;         /* rows * N or NULL */
  float* outY32;          /* rows * N or NULL */
  int32_t* alive_out;     /* rows: 1 if the row survived all layers */
  int32_t* dead_at;       /* rows: first layer index whose output was empty, L if none */
} plain_job;

static void* plain_worker(void* arg) {
  plain_job* j = (plain_job*)arg;
  const int N = j->N, L = j->L;
  double* a64 = NULL;
  double* y64 = NULL;
  float* a32 = NULL;
  float* y32 = NULL;
  if (j->precision == 64) {
    a64 = (double*)malloc(sizeof(double) * N);
    y64 = (double*)malloc(sizeof(double) * N);
  } else {
    a32 = (float*)malloc(sizeof(float) * N);
    y32 = (float*)malloc(sizeof(float) * N);
  }
  for (int64_t r = j->r0; r < j->r1; ++r) {
    const float* x = j->Y0 + r * (int64_t)N;
    int alive = 1, dead = L;
    if (j->precision == 64) {
      for (int c = 0; c < N; ++c) y64[c] = (double)x[c];
    } else {
      for (int c = 0; c < N; ++c) y32[c] = x[c];
    }
    for (int l = 0; l < L && alive; ++l) {
      const int32_t* ro = j->row_off + (int64_t)l * (N + 1);
      const int32_t* co = j->cols + j->nnz_off[l];
      const float* vo = j->vals + j->nnz_off[l];
      const float* bv = j->bias_vec ? j->bias_vec + (int64_t)l * N : NULL;
      int any = 0;
      if (j->precision == 64) {
        memset(a64, 0, sizeof(double) * N);
        for (int i = 0; i < N; ++i) {
          const double v = y64[i];
          if (v == 0.0) continue;
          for (int32_t k = ro[i]; k < ro[i + 1]; ++k) a64[co[k]] += v * (double)vo[k];
        }
        for (int c = 0; c < N; ++c) {
          const double b = bv ? (double)bv[c] : (double)j->bias;
          const double v = a64[c] + b;
          if (v > 0.0) any = 1;
          y64[c] = v < 0.0 ? 0.0 : (v > (double)j->clampv ? (double)j->clampv : v);
        }
      } else {
        memset(a32, 0, sizeof(float) * N);
        for (int i = 0; i < N; ++i) {
          const float v = y32[i];
          if (v == 0.f) continue;
          for (int32_t k = ro[i]; k < ro[i + 1]; ++k) {
            const float p = v * vo[k];
            a32[co[k]] = a32[co[k]] + p;
          }
        }
        for (int c = 0; c < N; ++c) {
          const float b = bv ? bv[c] : j->bias;
          const float v = a32[c] + b;
          if (v > 0.f) any = 1;
          y32[c] = v < 0.f ? 0.f : (v > j->clampv ? j->clampv : v);
        }
      }
      if (!any) {
        alive = 0;
        dead = l;
      }
    }
    if (!alive) {
      if (j->precision == 64) memset(y64, 0, sizeof(double) * N);
      else memset(y32, 0, sizeof(float) * N);
    }
    if (j->alive_out) j->alive_out[r] = alive;
    if (j->dead_at) j->dead_at[r] = dead;
    if (j->outY64) {
      double* o = j->outY64 + r * (int64_t)N;
      if (j->precision == 64) memcpy(o, y64, sizeof(double) * N);
      else
        for (int c = 0; c < N; ++c) o[c] = (double)y32[c];
    }
    if (j->outY32) {
      float* o = j->outY32 + r * (int64_t)N;
      if (j->precision == 64)
        for (int c = 0; c < N; ++c) o[c] = (float)y64[c];
      else memcpy(o, y32, sizeof(float) * N);
    }
  }
  free(a64);
  free(y64);
  free(a32);
  free(y32);
  return NULL;
}

/* Plain recurrence over rows [0, rows) with nthreads host threads. */
int oracle_infer(int N, int L, const int32_t* row_off, const int32_t* cols, const float* vals,
                 const int64_t* nnz_off, const float* bias_vec, float bias, float clampv,
                 const float* Y0, int64_t rows, int precision, int nthreads, double* outY64,
                 float* outY32, int32_t* alive_out, int32_t* dead_at) {
  if (N <= 0 || L < 0 || rows < 0 || !Y0 || (precision != 32 && precision != 64)) return 1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > rows && rows > 0) nthreads = (int)rows;
  if (rows == 0) return 0;
  plain_job* jobs = (plain_job*)calloc((size_t)nthreads, sizeof(plain_job));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  for (int t = 0; t < nthreads; ++t) {
    plain_job* j = &jobs[t];
    j->N = N;
    j->L = L;
    j->precision = precision;
    j->row_off = row_off;
    j->cols = cols;
    j->vals = vals;
    j->nnz_off = nnz_off;
    j->bias_vec = bias_vec;
    j->bias = bias;
    j->clampv = clampv;
    j->Y0 = Y0;
    j->r0 = rows * t / nthreads;
    j->r1 = rows * (t + 1) / nthreads;
    j->outY64 = outY64;
    j->outY32 = outY32;
    j->alive_out = alive_out;
    j->dead_at = dead_at;
    if (nthreads == 1) plain_worker(j);
    else pthread_create(&th[t], NULL, plain_worker, j);
  }
  if (nthreads > 1)
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
  return 0;
}

/* Category of each row from final activations (see header for the modes). */
int oracle_identify(const double* Y, int64_t rows, int N, int mode, int32_t* out) {
  for (int64_t r = 0; r < rows; ++r) {
    const double* y = Y + r * (int64_t)N;
    int flag = 0;
    if (mode == 0) {
      for (int c = 0; c < N && !flag; ++c) flag = y[c] > 0.0;
    } else {
      int acc = 0; /* int result, float binary op: acc = (int)((float)acc + y) */
      for (int c = 0; c < N; ++c) acc = (int)((float)acc + (float)y[c]);
      flag = acc > 0;
    }
    out[r] = flag;
  }
  return 0;
}

/* One FP64 layer for one row: out = W^T x (no bias), x dense. */
static void spmv64(int N, const int32_t* ro, const int32_t* co, const float* vo, const double* x,
                   double* out) {
  memset(out, 0, sizeof(double) * N);
  for (int i = 0; i < N; ++i) {
    const double v = x[i];
    if (v == 0.0) continue;
    for (int32_t k = ro[i]; k < ro[i + 1]; ++k) out[co[k]] += v * (double)vo[k];
  }
}
static double f64c(double v, double hi) { return v < 0.0 ? 0.0 : (v > hi ? hi : v); }

/*
 * SNICIT residue form in FP64 for rows [0, rows).  Layers [0, threshold) are
 * plain (dead rows leave); at the threshold every live row is assigned to the
 * nearest of the given centroid rows (which must be live; ncent >= 1) by L0
 * distance; layers [threshold, L) update centroids and residues; the result
 * is recovered.  outY (rows * N) receives recovered activations (zeros for
 * rows dead before the threshold), flags the categories (any > 0).
 * assign_out (rows, optional): centroid index per live row, -1 for dead rows;
 * nonempty_out (optional): number of non-empty residue rows at the threshold.
 */
int oracle_snicit(int N, int L, const int32_t* row_off, const int32_t* cols, const float* vals,
                  const int64_t* nnz_off, const float* bias_vec, float bias, float clampv,
                  const float* Y0, int64_t rows, int threshold, const int32_t* centroids,
                  int ncent, double* outY, int32_t* flags, int32_t* assign_out,
                  int64_t* nonempty_out) {
  if (threshold < 0) threshold = 0;
  if (threshold > L) threshold = L;
  const double hi = (double)clampv;
  double* Y = (double*)calloc((size_t)rows * N, sizeof(double));
  int32_t* live = (int32_t*)malloc(sizeof(int32_t) * (size_t)(rows > 0 ? rows : 1));
  double* acc = (double*)malloc(sizeof(double) * N);
  if (!Y || !live || !acc) return 2;
  for (int64_t r = 0; r < rows; ++r) {
    live[r] = 1;
    for (int c = 0; c < N; ++c) Y[r * N + c] = (double)Y0[r * N + c];
  }
  for (int l = 0; l < threshold; ++l) {
    const int32_t* ro = row_off + (int64_t)l * (N + 1);
    const int32_t* co = cols + nnz_off[l];
    const float* vo = vals + nnz_off[l];
    const float* bv = bias_vec ? bias_vec + (int64_t)l * N : NULL;
    for (int64_t r = 0; r < rows; ++r) {
      if (!live[r]) continue;
      double* y = Y + r * N;
      spmv64(N, ro, co, vo, y, acc);
      int any = 0;
      for (int c = 0; c < N; ++c) {
        const double v = acc[c] + (bv ? (double)bv[c] : (double)bias);
        if (v > 0.0) any = 1;
        y[c] = f64c(v, hi);
      }
      if (!any) {
        live[r] = 0;
        memset(y, 0, sizeof(double) * N);
      }
    }
  }
  if (threshold < L) {
    /* nearest centroid, residues */
    int32_t* cidx = (int32_t*)malloc(sizeof(int32_t) * (size_t)(rows > 0 ? rows : 1));
    int32_t* is_c = (int32_t*)calloc((size_t)(rows > 0 ? rows : 1), sizeof(int32_t));
    double* C = (double*)malloc(sizeof(double) * (size_t)ncent * N);
    double* P = (double*)malloc(sizeof(double) * (size_t)ncent * N);
    double* D = (double*)calloc((size_t)rows * N, sizeof(double));
    int32_t* ne = (int32_t*)calloc((size_t)(rows > 0 ? rows : 1), sizeof(int32_t));
    for (int k = 0; k < ncent; ++k) {
      is_c[centroids[k]] = 1;
      memcpy(C + (int64_t)k * N, Y + (int64_t)centroids[k] * N, sizeof(double) * N);
    }
    int64_t nonempty = 0;
    for (int64_t r = 0; r < rows; ++r) {
      cidx[r] = -1;
      if (!live[r]) continue;
      const double* y = Y + r * N;
      int best = N + 1, bk = 0;
      for (int k = 0; k < ncent; ++k) {
        const double* c = C + (int64_t)k * N;
        int d = 0;
        for (int i = 0; i < N; ++i) d += y[i] != c[i];
        if (d < best) {
          best = d;
          bk = k;
        }
      }
      if (is_c[r]) {
        for (int k = 0; k < ncent; ++k)
          if (centroids[k] == r) bk = k;
        best = 0;
      }
      cidx[r] = bk;
      if (!is_c[r] && best > 0) {
        ne[r] = 1;
        ++nonempty;
        for (int i = 0; i < N; ++i) D[r * N + i] = y[i] - C[(int64_t)bk * N + i];
      }
    }
    for (int l = threshold; l < L; ++l) {
      const int32_t* ro = row_off + (int64_t)l * (N + 1);
      const int32_t* co = cols + nnz_off[l];
      const float* vo = vals + nnz_off[l];
      const float* bv = bias_vec ? bias_vec + (int64_t)l * N : NULL;
      for (int k = 0; k < ncent; ++k) {
        double* c = C + (int64_t)k * N;
        double* p = P + (int64_t)k * N;
        spmv64(N, ro, co, vo, c, acc);
        for (int i = 0; i < N; ++i) {
          p[i] = acc[i] + (bv ? (double)bv[i] : (double)bias);
          c[i] = f64c(p[i], hi);
        }
      }
      for (int64_t r = 0; r < rows; ++r) {
        if (!ne[r]) continue;
        double* d = D + r * N;
        const double* p = P + (int64_t)cidx[r] * N;
        spmv64(N, ro, co, vo, d, acc);
        int any = 0;
        for (int i = 0; i < N; ++i) {
          d[i] = f64c(p[i] + acc[i], hi) - f64c(p[i], hi);
          if (d[i] != 0.0) any = 1;
        }
        if (!any) ne[r] = 0;
      }
    }
    for (int64_t r = 0; r < rows; ++r) {
      double* y = Y + r * N;
      if (!live[r]) continue;
      const double* c = C + (int64_t)cidx[r] * N;
      for (int i = 0; i < N; ++i) y[i] = c[i] + (ne[r] ? D[r * N + i] : 0.0);
    }
    if (assign_out)
      for (int64_t r = 0; r < rows; ++r) assign_out[r] = cidx[r];
    if (nonempty_out) *nonempty_out = nonempty;
    free(cidx);
    free(is_c);
    free(C);
    free(P);
    free(D);
    free(ne);
  }
  for (int64_t r = 0; r < rows; ++r) {
    int any = 0;
    for (int i = 0; i < N && !any; ++i) any = Y[r * N + i] > 0.0;
    if (flags) flags[r] = any;
  }
  if (outY) memcpy(outY, Y, sizeof(double) * (size_t)rows * N);
  free(Y);
  free(live);
  free(acc);
  return 0;
}

/*
 * The reference's centroid candidates: the first `sample` rows of the live
 * set (indices into `Ylive`, a live-rows-only matrix), binned as reduction()
 * does with blockDim = (1024/16, 16): bin b sums positions [64b, 64b + N/16)
 * (overlapping for N > 1024), then pruned greedily: candidate j is dropped
 * when another kept candidate has no bin differing by more than 0.03.
 * Writes kept candidate indices to out (in order) and returns their count.
 */
int oracle_ref_candidates(const float* Ylive, int64_t live_rows, int N, int sample, int32_t* out) {
  if (sample > 32) sample = 32;
  if (sample > live_rows) sample = (int)live_rows;
  float bins[32][16];
  for (int s = 0; s < sample; ++s)
    for (int b = 0; b < 16; ++b) {
      float sum = 0.f;
      for (int r = 0; r < N / 16; ++r) sum += Ylive[(int64_t)s * N + b * 64 + r];
      bins[s][b] = sum;
    }
  int keep[32];
  for (int s = 0; s < sample; ++s) keep[s] = 1;
  for (int cmp = 0; cmp < sample; ++cmp) {
    if (!keep[cmp]) continue;
    for (int s = 0; s < sample; ++s) {
      if (s == cmp || !keep[s]) continue;
      int diff = 0;
      for (int b = 0; b < 16; ++b)
        if (fabsf(bins[s][b] - bins[cmp][b]) > 0.03f) ++diff;
      if ((float)diff < 16.f * 0.03f) keep[s] = 0;
    }
  }
  int n = 0;
  for (int s = 0; s < sample; ++s)
    if (keep[s]) out[n++] = s;
  return n;
}

#ifdef __cplusplus
}
#endif
