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
 *   oracle_gen_*       restatement of the synthetic SDGC data (counter-based
 *                      SplitMix64 streams keyed by (seed, kind, layer/row), Steele
 *                      et al., OOPSLA 2014): the same rows and weight columns as the
 *                      engine's own generator, so the CPU baseline and the
 *                      reference arm of the benchmark need nothing from the product.
 *   oracle_port_stream the FP32 port of bf_inference (same arithmetic as
 *                      oracle_infer precision 32) over row groups with the
 *                      synthetic weights generated layer by layer, so a
 *                      1920-layer net never sits in host memory whole; per group
 *                      it times the layer arithmetic only (not the weight
 *                      generation), like the reference's own timers around the
 *                      layer loop (src/SDGC/BF/BF.hpp:159,217-219).
 *   oracle_infer_stream64   the FP64 oracle of the synthetic net with the
 *                      weights generated layer by layer (the 1920-layer nets'
 *                      weights are 32 GB as CSR; this holds one layer).
 *
 * Parity pins: the golden fixtures under tests/golden/ (outputs of the
 * reference's own bf_inference / snig_inference kernels, compiled from its
 * sources and run on a GB300) are checked against oracle_infer by the CPU
 * tests.
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <pthread.h>
#include <time.h>
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

/* ---- synthetic data (restatement of the engine's generator) ------------- */

static uint64_t sm_fin(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
#define SM_GOLDEN 0x9E3779B97F4A7C15ull
static uint64_t sm_key(uint64_t seed, uint64_t kind, uint64_t a, uint64_t b) {
  uint64_t k = sm_fin(seed + SM_GOLDEN);
  k = sm_fin(k ^ (kind * 0xD1B54A32D192ED03ull + SM_GOLDEN));
  k = sm_fin(k ^ (a * 0xABC98388FB8FAC03ull + SM_GOLDEN));
  k = sm_fin(k ^ (b * 0x8CB92BA72F3D8DD7ull + SM_GOLDEN));
  return k;
}
static uint64_t sm_draw(uint64_t key, uint64_t i) { return sm_fin(key + (i + 1) * SM_GOLDEN); }
/* high 64 bits of u * n, from 32-bit halves (no 128-bit type needed) */
static uint32_t sm_bounded(uint64_t u, uint32_t n) {
  const uint64_t lo = (u & 0xffffffffull) * n, hi = (u >> 32) * n;
  return (uint32_t)((hi + (lo >> 32)) >> 32);
}
static double sm_unit53(uint64_t u) { return (double)(u >> 11) * (1.0 / 9007199254740992.0); }
static int cmp_u64(const void* a, const void* b) {
  const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* Columns of input row `row` of `layer`: nnz distinct outputs in draw order. */
static void gen_row_cols(uint64_t seed, int layer, int row, int N, int nnz, int32_t* cols) {
  const uint64_t key = sm_key(seed, 1, (uint64_t)layer, (uint64_t)row);
  int have = 0;
  for (uint64_t i = 0; have < nnz; ++i) {
    const int32_t c = (int32_t)sm_bounded(sm_draw(key, i), (uint32_t)N);
    int dup = 0;
    for (int k = 0; k < have; ++k)
      if (cols[k] == c) {
        dup = 1;
        break;
      }
    if (!dup) cols[have++] = c;
  }
}

/* Seeded 0/1 input rows [row_offset, row_offset + rows): row density
 * 0.95 * (2nd smallest of 9 uniforms), entries 1 with that probability. */
int oracle_gen_inputs(int N, uint64_t seed, int64_t row_offset, int64_t rows, float* out) {
  if (N <= 0 || rows < 0 || row_offset < 0 || (!out && rows > 0)) return 1;
  for (int64_t r = 0; r < rows; ++r) {
    const uint64_t key = sm_key(seed, 2, 0, (uint64_t)(row_offset + r));
    uint64_t u[9];
    for (int i = 0; i < 9; ++i) u[i] = sm_draw(key, (uint64_t)i) >> 11;
    qsort(u, 9, sizeof(uint64_t), cmp_u64);
    const double rho = 0.95 * ((double)u[1] * (1.0 / 9007199254740992.0));
    float* o = out + r * (int64_t)N;
    for (int j = 0; j < N; ++j) o[j] = sm_unit53(sm_draw(key, 9 + (uint64_t)j)) < rho ? 1.f : 0.f;
  }
  return 0;
}

/* One synthetic layer as CSR by input row: row_off[N+1], cols/vals N*nnz
 * (columns in draw order; all distinct, so no duplicates to sum). */
int oracle_gen_layer_csr(int N, uint64_t seed, int layer, int nnz, float value, int32_t* row_off,
                         int32_t* cols, float* vals) {
  if (N <= 0 || nnz <= 0 || nnz > N || layer < 0) return 1;
  for (int i = 0; i <= N; ++i) row_off[i] = i * nnz;
  for (int i = 0; i < N; ++i) {
    gen_row_cols(seed, layer, i, N, nnz, cols + (int64_t)i * nnz);
    for (int k = 0; k < nnz; ++k) vals[(int64_t)i * nnz + k] = value;
  }
  return 0;
}

/* RadiX-Net layer, radix 2 with dense blocks of `block` neurons (Robinett and
 * Kepner, 2019): N = block * M, M = 2^k nodes, neuron v = (v / M, node v % M).
 * Stated output by output -- output (r, c) reads every input of nodes c and
 * c + 2^(layer mod k) (mod M), the windows the reference's XY kernels read
 * after its HashReorder (src/SDGC/XY/kernel.hpp:71-91, strides from
 * src/SDGC/SNICIT/SNICIT.hpp:329-342) -- then turned into CSR by input row
 * (outputs ascending). */
int oracle_gen_radixnet_csr(int N, int block, int layer, float value, int32_t* row_off,
                            int32_t* cols, float* vals) {
  if (block < 1 || N < 2 * block || N % block != 0 || layer < 0) return 1;
  const int M = N / block;
  if (M & (M - 1)) return 1;
  int k = 0;
  while ((1 << k) < M) ++k;
  const int step = 1 << (layer % k);
  for (int i = 0; i <= N; ++i) row_off[i] = 0;
  for (int out = 0; out < N; ++out) {
    const int nodes[2] = {out % M, (out % M + step) % M};
    for (int n = 0; n < 2; ++n)
      for (int r = 0; r < block; ++r) row_off[r * M + nodes[n] + 1]++;
  }
  for (int i = 0; i < N; ++i) row_off[i + 1] += row_off[i];
  int32_t* cur = (int32_t*)malloc(sizeof(int32_t) * (size_t)N);
  if (!cur) return 1;
  for (int i = 0; i < N; ++i) cur[i] = row_off[i];
  for (int out = 0; out < N; ++out) {
    const int nodes[2] = {out % M, (out % M + step) % M};
    for (int n = 0; n < 2; ++n)
      for (int r = 0; r < block; ++r) {
        const int in = r * M + nodes[n];
        cols[cur[in]] = out;
        vals[cur[in]++] = value;
      }
  }
  free(cur);
  return 0;
}

/* ---- FP32 port over groups of rows, weights generated layer by layer ---- */

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

typedef struct {
  int N, L, nnz, ngroups, nthreads;
  uint64_t seed;
  float wval, bias, clampv;
  float* ybuf[2];           /* rows * N each: layer l reads ybuf[l & 1], writes the other */
  int64_t rows;
  const int64_t* group_off; /* ngroups + 1 row offsets */
  int32_t* live;            /* rows: alive before the current layer */
  int32_t* live_next;       /* rows: some output > 0 in the current layer */
  int32_t* cols;            /* N * nnz out-edges of the current layer, by input */
  int32_t* tin_off;         /* N + 1: in-edges of every output ... */
  int32_t* tin;             /* N * nnz ... inputs ascending */
  int64_t* tot;             /* nthreads: edges per thread's output range */
  int32_t* cnt;             /* nthreads * N: per-thread edge counts, then positions */
  int64_t next;             /* work counter of the current phase */
  double* secs;             /* ngroups */
  pthread_barrier_t bar;
} stream_job;

typedef struct {
  stream_job* j;
  int t;
} stream_arg;

enum { kPortBlock = 4096 };  /* outputs per work item */

static void* stream_worker(void* p) {
  stream_arg* a = (stream_arg*)p;
  stream_job* j = a->j;
  const int N = j->N, nnz = j->nnz, T = j->nthreads;
  const int c0 = (int)((int64_t)N * a->t / T), c1 = (int)((int64_t)N * (a->t + 1) / T);
  const int nblk = (N + kPortBlock - 1) / kPortBlock;
  for (int l = 0; l < j->L; ++l) {
    const float* yin_all = j->ybuf[l & 1];
    float* yout_all = j->ybuf[(l + 1) & 1];
    /* weights of layer l: input rows split over the threads, then the
       in-edges of every output (inputs ascending), outputs split over the
       threads (untimed) */
    for (int i = (int)((int64_t)N * a->t / T); i < (int)((int64_t)N * (a->t + 1) / T); ++i)
      gen_row_cols(j->seed, l, i, N, nnz, j->cols + (int64_t)i * nnz);
    pthread_barrier_wait(&j->bar);
    {
      /* in-edges by output, inputs ascending: thread t counts the edges of its
         input range per output (cnt row t), the output ranges turn the counts
         into positions (outputs in order, then threads in order, so that the
         inputs of an output stay ascending), and each thread places its edges */
      const int i0 = (int)((int64_t)N * a->t / T), i1 = (int)((int64_t)N * (a->t + 1) / T);
      int32_t* mycnt = j->cnt + (int64_t)a->t * N;
      memset(mycnt, 0, sizeof(int32_t) * (size_t)N);
      for (int64_t e = (int64_t)i0 * nnz; e < (int64_t)i1 * nnz; ++e) mycnt[j->cols[e]]++;
      pthread_barrier_wait(&j->bar);
      int64_t mine = 0;
      for (int c = c0; c < c1; ++c)
        for (int t = 0; t < T; ++t) mine += j->cnt[(int64_t)t * N + c];
      j->tot[a->t] = mine;
      pthread_barrier_wait(&j->bar);
      int64_t run = 0;
      for (int t = 0; t < a->t; ++t) run += j->tot[t];
      for (int c = c0; c < c1; ++c) {
        j->tin_off[c] = (int32_t)run;
        for (int t = 0; t < T; ++t) {
          const int32_t n = j->cnt[(int64_t)t * N + c];
          j->cnt[(int64_t)t * N + c] = (int32_t)run;  /* thread t's first position for c */
          run += n;
        }
      }
      if (a->t == T - 1) j->tin_off[N] = (int32_t)run;
      pthread_barrier_wait(&j->bar);
      for (int i = i0; i < i1; ++i)
        for (int k = 0; k < nnz; ++k) j->tin[mycnt[j->cols[(int64_t)i * nnz + k]]++] = i;
    }
    for (int64_t r = (j->rows * a->t) / T; r < (j->rows * (a->t + 1)) / T; ++r) j->live_next[r] = 0;
    pthread_barrier_wait(&j->bar);
    for (int g = 0; g < j->ngroups; ++g) {
      double t0 = 0.0;
      const int64_t g0 = j->group_off[g], items = (j->group_off[g + 1] - g0) * nblk;
      if (a->t == 0) {
        __atomic_store_n(&j->next, 0, __ATOMIC_SEQ_CST);
        t0 = now_s();
      }
      pthread_barrier_wait(&j->bar);
      for (;;) {
        const int64_t it = __atomic_fetch_add(&j->next, 1, __ATOMIC_SEQ_CST);
        if (it >= items) break;
        const int64_t r = g0 + it / nblk;
        if (!j->live[r]) continue;
        const int b0 = (int)(it % nblk) * kPortBlock, b1 = b0 + kPortBlock < N ? b0 + kPortBlock : N;
        const float* y = yin_all + r * (int64_t)N;
        float* yo = yout_all + r * (int64_t)N;
        int any = 0;
        /* each output sums its nonzero inputs in ascending order, products
           first: the arithmetic of the input-major scatter of oracle_infer */
        for (int c = b0; c < b1; ++c) {
          float acc = 0.f;
          for (int32_t e = j->tin_off[c]; e < j->tin_off[c + 1]; ++e) {
            const float v = y[j->tin[e]];
            if (v == 0.f) continue;
            const float prod = v * j->wval;
            acc = acc + prod;
          }
          const float v = acc + j->bias;
          if (v > 0.f) any = 1;
          yo[c] = v < 0.f ? 0.f : (v > j->clampv ? j->clampv : v);
        }
        if (any) __atomic_store_n(&j->live_next[r], 1, __ATOMIC_RELAXED);
      }
      pthread_barrier_wait(&j->bar);
      if (a->t == 0) j->secs[g] += now_s() - t0;
    }
    for (int64_t r = (j->rows * a->t) / T; r < (j->rows * (a->t + 1)) / T; ++r)
      j->live[r] = j->live[r] && j->live_next[r];
    pthread_barrier_wait(&j->bar);
  }
  return NULL;
}

/* FP32 plain recurrence (the arithmetic of oracle_infer precision 32) of the
 * synthetic net (seed, nnz distinct columns per input row, every value wval,
 * scalar bias) over the rows of Y (rows x N, overwritten with the final
 * activations).  Rows [group_off[g], group_off[g+1]) form group g; secs[g]
 * receives the wall time of group g's layer arithmetic summed over the
 * layers (all threads on one group at a time: a work item is a row's block of
 * 4096 outputs, so the threads stay busy when only a few rows are left alive).
 * alive_out[r] = 1 if row r survives every layer. */
int oracle_port_stream(int N, int L, uint64_t seed, int nnz, float wval, float bias, float clampv,
                       float* Y, int64_t rows, const int64_t* group_off, int ngroups,
                       int nthreads, int32_t* alive_out, double* secs) {
  if (N <= 0 || L < 0 || nnz <= 0 || nnz > N || !Y || rows < 0 || ngroups <= 0 || !group_off ||
      group_off[0] != 0 || group_off[ngroups] != rows || !secs)
    return 1;
  if (nthreads < 1) nthreads = 1;
  stream_job j;
  memset(&j, 0, sizeof(j));
  j.N = N;
  j.L = L;
  j.nnz = nnz;
  j.ngroups = ngroups;
  j.nthreads = nthreads;
  j.seed = seed;
  j.wval = wval;
  j.bias = bias;
  j.clampv = clampv;
  j.rows = rows;
  j.group_off = group_off;
  j.secs = secs;
  const size_t ysz = sizeof(float) * (size_t)(rows > 0 ? rows : 1) * (size_t)N;
  j.ybuf[0] = Y;
  j.ybuf[1] = (float*)malloc(ysz);
  j.live = (int32_t*)malloc(sizeof(int32_t) * (size_t)(rows > 0 ? rows : 1));
  j.live_next = (int32_t*)malloc(sizeof(int32_t) * (size_t)(rows > 0 ? rows : 1));
  j.cols = (int32_t*)malloc(sizeof(int32_t) * (size_t)N * (size_t)nnz);
  j.tin = (int32_t*)malloc(sizeof(int32_t) * (size_t)N * (size_t)nnz);
  j.tin_off = (int32_t*)malloc(sizeof(int32_t) * (size_t)(N + 1));
  j.tot = (int64_t*)calloc((size_t)nthreads, sizeof(int64_t));
  j.cnt = (int32_t*)malloc(sizeof(int32_t) * (size_t)nthreads * (size_t)N);
  /* every row enters layer 0 (an all-zero row dies there, BF.hpp:222-229) */
  for (int64_t r = 0; r < rows; ++r) j.live[r] = 1;
  for (int g = 0; g < ngroups; ++g) secs[g] = 0.0;
  pthread_barrier_init(&j.bar, NULL, (unsigned)nthreads);
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  stream_arg* args = (stream_arg*)calloc((size_t)nthreads, sizeof(stream_arg));
  for (int t = 0; t < nthreads; ++t) {
    args[t].j = &j;
    args[t].t = t;
    if (t > 0) pthread_create(&th[t], NULL, stream_worker, &args[t]);
  }
  stream_worker(&args[0]);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
  pthread_barrier_destroy(&j.bar);
  const float* fin = j.ybuf[L & 1];
  for (int64_t r = 0; r < rows; ++r) {
    if (alive_out) alive_out[r] = j.live[r];
    if (!j.live[r]) memset(Y + r * (int64_t)N, 0, sizeof(float) * (size_t)N);
    else if (fin != Y) memcpy(Y + r * (int64_t)N, fin + r * (int64_t)N, sizeof(float) * (size_t)N);
  }
  free(th);
  free(args);
  free(j.ybuf[1]);
  free(j.live);
  free(j.live_next);
  free(j.cols);
  free(j.tin);
  free(j.tin_off);
  free(j.tot);
  free(j.cnt);
  return 0;
}

/* ---- FP64 oracle with the weights generated layer by layer -------------- */

typedef struct {
  int N, L, nnz, nthreads;
  uint64_t seed;
  double wval, bias, clampv;
  double* y;       /* rows * N */
  int64_t rows;
  int32_t* live;
  int32_t* cols;
  int64_t next;
  pthread_barrier_t bar;
} stream64_job;

static void* stream64_worker(void* p) {
  stream_arg* a = (stream_arg*)p;
  stream64_job* j = (stream64_job*)a->j;
  const int N = j->N, nnz = j->nnz, T = j->nthreads;
  double* acc = (double*)malloc(sizeof(double) * (size_t)N);
  for (int l = 0; l < j->L; ++l) {
    for (int i = (int)((int64_t)N * a->t / T); i < (int)((int64_t)N * (a->t + 1) / T); ++i)
      gen_row_cols(j->seed, l, i, N, nnz, j->cols + (int64_t)i * nnz);
    if (a->t == 0) __atomic_store_n(&j->next, 0, __ATOMIC_SEQ_CST);
    pthread_barrier_wait(&j->bar);
    for (;;) {
      const int64_t r = __atomic_fetch_add(&j->next, 1, __ATOMIC_SEQ_CST);
      if (r >= j->rows) break;
      if (!j->live[r]) continue;
      double* y = j->y + r * (int64_t)N;
      memset(acc, 0, sizeof(double) * (size_t)N);
      for (int i = 0; i < N; ++i) {
        const double v = y[i];
        if (v == 0.0) continue;
        const int32_t* co = j->cols + (int64_t)i * nnz;
        for (int k = 0; k < nnz; ++k) acc[co[k]] += v * j->wval;
      }
      int any = 0;
      for (int c = 0; c < N; ++c) {
        const double v = acc[c] + j->bias;
        if (v > 0.0) any = 1;
        y[c] = v < 0.0 ? 0.0 : (v > j->clampv ? j->clampv : v);
      }
      if (!any) j->live[r] = 0;
    }
    pthread_barrier_wait(&j->bar);
  }
  free(acc);
  return NULL;
}

/* The FP64 oracle (oracle_infer precision 64 arithmetic) of the synthetic
 * net, weights generated layer by layer: Y64 (rows x N) receives the final
 * activations (zero rows for dead samples), alive_out the categories. */
int oracle_infer_stream64(int N, int L, uint64_t seed, int nnz, float wval, float bias,
                          float clampv, const float* Y0, int64_t rows, int nthreads, double* Y64,
                          int32_t* alive_out) {
  if (N <= 0 || L < 0 || nnz <= 0 || nnz > N || !Y0 || rows < 0 || !Y64) return 1;
  if (nthreads < 1) nthreads = 1;
  stream64_job j;
  memset(&j, 0, sizeof(j));
  j.N = N;
  j.L = L;
  j.nnz = nnz;
  j.nthreads = nthreads;
  j.seed = seed;
  j.wval = (double)wval;
  j.bias = (double)bias;
  j.clampv = (double)clampv;
  j.y = Y64;
  j.rows = rows;
  for (int64_t i = 0; i < rows * (int64_t)N; ++i) Y64[i] = (double)Y0[i];
  j.live = (int32_t*)malloc(sizeof(int32_t) * (size_t)(rows > 0 ? rows : 1));
  j.cols = (int32_t*)malloc(sizeof(int32_t) * (size_t)N * (size_t)nnz);
  for (int64_t r = 0; r < rows; ++r) j.live[r] = 1;
  pthread_barrier_init(&j.bar, NULL, (unsigned)nthreads);
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  stream_arg* args = (stream_arg*)calloc((size_t)nthreads, sizeof(stream_arg));
  for (int t = 0; t < nthreads; ++t) {
    args[t].j = (stream_job*)&j;
    args[t].t = t;
    if (t > 0) pthread_create(&th[t], NULL, stream64_worker, &args[t]);
  }
  stream64_worker(&args[0]);
  for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
  pthread_barrier_destroy(&j.bar);
  for (int64_t r = 0; r < rows; ++r) {
    if (alive_out) alive_out[r] = j.live[r];
    if (!j.live[r]) memset(Y64 + r * (int64_t)N, 0, sizeof(double) * (size_t)N);
  }
  free(th);
  free(args);
  free(j.live);
  free(j.cols);
  return 0;
}

#ifdef __cplusplus
}
#endif
