/*
 * CPU ORACLE for the Jaccard hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the algorithm of the reference's SYCL kernels so that the
 * GPU engine's results can be checked against it.  It is imported only by the tests, by
 * the smoke check of the build entry point and by the CPU-baseline leg of the benchmark.
 * Nothing in the engine links against it.
 *
 * Reference files (vtsynergy/SYCL-Jaccard):
 *   - jaccard.cpp:53-137   parallel_prefix_sum: 32-wide Hillis-Steele scan with a carry
 *   - jaccard.cpp:236-261  Jaccard_RowSumKernel::operator()
 *   - jaccard.cpp:150-159  FillKernel::operator()
 *   - jaccard.cpp:315-400  Jaccard_IsKernel::operator()  (weighted / unweighted)
 *   - jaccard.cpp:402-418  Jaccard_IsKernel::invoke launch shape {8 rows, 4 j-lanes, 8 i-lanes}
 *   - jaccard.cpp:608-620  Jaccard_JwKernel::operator()
 *   - jaccard.cpp:654-664  Jaccard_ec_scan::operator()
 *   - jaccard.cpp:703-743  Jaccard_ec_unweighted::operator()
 *   - jaccard.cpp:784-899  detail::jaccard (EC / VC sequencing)
 *
 * Order of floating-point accumulation.  The reference adds into weight_i[j] with atomic
 * adds from 8 "i-lanes" (jaccard.cpp:343, 370-396); when the work-items of a group execute
 * one after another in linear-id order (a CPU SYCL device), lane 0 adds all of its matches
 * (ref positions 0, 8, 16, ...) first, then lane 1 (positions 1, 9, ...), and so on.  This
 * oracle reproduces exactly that order, which is also the order of the reference compiled
 * against the host SYCL subset in oracle/syclshim.
 *
 * Entry points are row- or edge-parallel with OpenMP; results do not depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define JXO_IS_I_LANES 8 /* jaccard.cpp:409,414: local range {8, y=4, 32/y=8} */
#define JXO_IS_J_LANES 4
#define JXO_WARP 32 /* jaccard.cpp:272: RowSum local range {1, 32} */

static void jxo_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/*
 * Row sum of one row, jaccard.cpp:53-137 with blockDim.x = 32.
 * Per 32-element chunk the lanes run an inclusive Hillis-Steele scan (steps 1,2,4,8,16,
 * jaccard.cpp:101-117), then add the carry `last` (lane 31 of the previous chunk,
 * jaccard.cpp:92,119).  The row total is lane 31's value after the last chunk
 * (jaccard.cpp:131-136).  Lanes past the row end contribute 0.0 (jaccard.cpp:98).
 */
static float jxo_row_prefix_total(int32_t start, int32_t len, const int32_t *ind, const float *w) {
  float sum[JXO_WARP];
  float tmp[JXO_WARP];
  for (int k = 0; k < JXO_WARP; ++k) sum[k] = 0.0f;
  const int32_t mn = ((len + JXO_WARP - 1) / JXO_WARP) * JXO_WARP;
  for (int32_t i0 = 0; i0 < mn; i0 += JXO_WARP) {
    const float last = sum[JXO_WARP - 1];
    for (int k = 0; k < JXO_WARP; ++k) sum[k] = (i0 + k < len) ? w[ind[start + i0 + k]] : 0.0f;
    for (int j = 1; j < JXO_WARP; j *= 2) {
      for (int k = 0; k < JXO_WARP; ++k) tmp[k] = sum[k];
      for (int k = j; k < JXO_WARP; ++k) sum[k] += tmp[k - j];
    }
    for (int k = 0; k < JXO_WARP; ++k) sum[k] += last;
  }
  return sum[JXO_WARP - 1];
}

/*
 * Jaccard_RowSumKernel (jaccard.cpp:236-261): work[row] = (float)deg (unweighted, w == NULL)
 * or the prefix-sum total of w[ind[k]] over the row (weighted).
 */
void jxo_rowsum(int32_t n, const int32_t *row_ptr, const int32_t *ind, const float *w,
                float *work, int nthreads) {
  jxo_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t row = 0; row < n; ++row) {
    const int32_t start = row_ptr[row], len = row_ptr[row + 1] - row_ptr[row];
    work[row] = w ? jxo_row_prefix_total(start, len, ind, w) : (float)len;
  }
}

/* FillKernel (jaccard.cpp:150-159). */
void jxo_fill(int64_t n, float *x, float value) {
  for (int64_t i = 0; i < n; ++i) x[i] = value;
}

/* Binary search of `key` in ind[lo .. hi] (inclusive), jaccard.cpp:353-367. */
static inline int jxo_found(const int32_t *ind, int32_t left, int32_t right, int32_t key) {
  while (left <= right) {
    const int32_t middle = (left + right) >> 1;
    const int32_t cur_col = ind[middle];
    if (cur_col > key)
      right = middle - 1;
    else if (cur_col < key)
      left = middle + 1;
    else
      return 1;
  }
  return 0;
}

/* Row of stored edge j, r0 <= row < r1 (the last row whose offset is <= j). */
static inline int32_t jxo_row_of(const int32_t *row_ptr, int32_t r0, int32_t r1, int64_t j) {
  int32_t lo = r0, hi = r1 - 1;
  while (lo < hi) {
    const int32_t mid = lo + (hi - lo + 1) / 2;
    if ((int64_t)row_ptr[mid] <= j) lo = mid; else hi = mid - 1;
  }
  return lo;
}

/*
 * Jaccard_IsKernel (jaccard.cpp:315-400) for rows [r0, r1):
 *   weight_s[j]  = work[row] + work[col]                         (jaccard.cpp:339)
 *   weight_i[j] += ref_val for every ref element found in cur     (jaccard.cpp:343-396)
 * ref is the shorter list, ties go to col (jaccard.cpp:333-336).  weight_i accumulates onto
 * its current contents (the reference fills it with 0 first, jaccard.cpp:836).
 */
void jxo_intersect_rows(int32_t r0, int32_t r1, const int32_t *row_ptr, const int32_t *ind,
                        const float *w, const float *work, float *weight_i, float *weight_s,
                        int nthreads) {
  jxo_threads(nthreads);
  /* edge-parallel (a hub row spreads over the threads); each edge's sum is sequential */
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t j = row_ptr[r0]; j < (int64_t)row_ptr[r1]; ++j) {
    const int32_t row = jxo_row_of(row_ptr, r0, r1, j);
    const int32_t col = ind[j];
    const int32_t Ni = row_ptr[row + 1] - row_ptr[row];
    const int32_t Nj = row_ptr[col + 1] - row_ptr[col];
    const int32_t ref = (Ni < Nj) ? row : col;
    const int32_t cur = (Ni < Nj) ? col : row;
    if (weight_s) weight_s[j] = work[row] + work[col];
    float acc = weight_i[j];
    for (int il = 0; il < JXO_IS_I_LANES; ++il) {
      for (int32_t i = row_ptr[ref] + il; i < row_ptr[ref + 1]; i += JXO_IS_I_LANES) {
        const int32_t ref_col = ind[i];
        const float ref_val = w ? w[ref_col] : 1.0f;
        if (jxo_found(ind, row_ptr[cur], row_ptr[cur + 1] - 1, ref_col)) acc = ref_val + acc;
      }
    }
    weight_i[j] = acc;
  }
}

/* Jaccard_JwKernel (jaccard.cpp:608-620): weight_j = Wi / (Ws - Wi). */
void jxo_weight(int64_t e, const float *weight_i, const float *weight_s, float *weight_j) {
  for (int64_t j = 0; j < e; ++j) {
    const float Wi = weight_i[j], Ws = weight_s[j];
    const float Wu = Ws - Wi;
    weight_j[j] = Wi / Wu;
  }
}

/* Jaccard_ec_scan (jaccard.cpp:654-664): dest_ind[k] = row, weight_j[k] = 0. */
void jxo_ec_scan(int32_t n, const int32_t *row_ptr, int32_t *dest_ind, float *weight_j) {
  for (int32_t row = 0; row < n; ++row)
    for (int32_t i = row_ptr[row]; i < row_ptr[row + 1]; ++i) {
      dest_ind[i] = row;
      weight_j[i] = 0.0f;
    }
}

/*
 * Jaccard_ec_unweighted (jaccard.cpp:703-743) for edges [e0, e1):
 * row = csrInd[tid] (the neighbour), col = dest_ind[tid] (the source row); ref is the shorter
 * list with ties going to col (jaccard.cpp:717-719); each match adds 1 to weight_j[tid]
 * (jaccard.cpp:735); J = c / ((float)(Ni + Nj) - c) (jaccard.cpp:741).
 */
void jxo_ec_edges(int64_t e0, int64_t e1, const int32_t *row_ptr, const int32_t *ind,
                  const int32_t *dest_ind, float *weight_j, int nthreads) {
  jxo_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t tid = e0; tid < e1; ++tid) {
    const int32_t row = ind[tid];
    const int32_t col = dest_ind[tid];
    const int32_t Ni = row_ptr[row + 1] - row_ptr[row];
    const int32_t Nj = row_ptr[col + 1] - row_ptr[col];
    const int32_t ref = (Ni < Nj) ? row : col;
    const int32_t cur = (Ni < Nj) ? col : row;
    float c = weight_j[tid];
    for (int32_t i = row_ptr[ref]; i < row_ptr[ref + 1]; ++i)
      if (jxo_found(ind, row_ptr[cur], row_ptr[cur + 1] - 1, ind[i])) c = c + 1.0f;
    weight_j[tid] = c / ((float)(Ni + Nj) - c);
  }
}

/*
 * detail::jaccard (jaccard.cpp:784-899) restricted to the edges of rows [r0, r1), written
 * into out[row_ptr[r0] .. row_ptr[r1]).  ec != 0 runs the edge-centric path (weights are
 * ignored, as jaccard.cpp:790 does); otherwise RowSum -> Fill -> IS -> JW.
 * `work` (n floats) may be passed in precomputed; when NULL it is computed here.
 */
int jxo_jaccard_rows(int ec, int32_t n, const int32_t *row_ptr, const int32_t *ind,
                     const float *w, int32_t r0, int32_t r1, const float *work_in, float *out,
                     int nthreads) {
  const int64_t base = row_ptr[r0];
  const int64_t cnt = (int64_t)row_ptr[r1] - base;
  if (ec) {
    int32_t *dest = (int32_t *)malloc(sizeof(int32_t) * (cnt > 0 ? cnt : 1));
    float *wj = (float *)malloc(sizeof(float) * (cnt > 0 ? cnt : 1));
    if (!dest || !wj) {
      free(dest);
      free(wj);
      return -1;
    }
    for (int32_t row = r0; row < r1; ++row)
      for (int32_t i = row_ptr[row]; i < row_ptr[row + 1]; ++i) {
        dest[i - base] = row;
        wj[i - base] = 0.0f;
      }
    /* jxo_ec_edges indexes absolute edge ids: offset the arrays. */
    jxo_ec_edges(base, base + cnt, row_ptr, ind, dest - base, wj - base, nthreads);
    memcpy(out, wj, sizeof(float) * cnt);
    free(dest);
    free(wj);
    return 0;
  }
  float *work = (float *)work_in;
  float *own = NULL;
  if (!work) {
    own = (float *)malloc(sizeof(float) * (n > 0 ? n : 1));
    if (!own) return -1;
    jxo_rowsum(n, row_ptr, ind, w, own, nthreads);
    work = own;
  }
  float *wi = (float *)calloc(cnt > 0 ? cnt : 1, sizeof(float));
  float *ws = (float *)malloc(sizeof(float) * (cnt > 0 ? cnt : 1));
  if (!wi || !ws) {
    free(own);
    free(wi);
    free(ws);
    return -1;
  }
  jxo_intersect_rows(r0, r1, row_ptr, ind, w, work, wi - base, ws - base, nthreads);
  jxo_weight(cnt, wi, ws, out);
  free(own);
  free(wi);
  free(ws);
  return 0;
}

/* Whole-graph convenience form of jxo_jaccard_rows. */
int jxo_jaccard(int ec, int32_t n, const int32_t *row_ptr, const int32_t *ind, const float *w,
                float *out, int nthreads) {
  return jxo_jaccard_rows(ec, n, row_ptr, ind, w, 0, n, NULL, out, nthreads);
}

/*
 * Intersection counts |N(u) n N(v)| per stored edge (the integer core of both paths) for
 * rows [r0, r1), written to cnt[row_ptr[r0] ..].
 */
void jxo_counts_rows(int32_t r0, int32_t r1, const int32_t *row_ptr, const int32_t *ind,
                     int32_t *cnt, int nthreads) {
  jxo_threads(nthreads);
  const int64_t base = row_ptr[r0];
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t j = base; j < (int64_t)row_ptr[r1]; ++j) {
    const int32_t row = jxo_row_of(row_ptr, r0, r1, j);
    const int32_t col = ind[j];
    const int32_t Ni = row_ptr[row + 1] - row_ptr[row];
    const int32_t Nj = row_ptr[col + 1] - row_ptr[col];
    const int32_t ref = (Ni < Nj) ? row : col;
    const int32_t cur = (Ni < Nj) ? col : row;
    int32_t c = 0;
    for (int32_t i = row_ptr[ref]; i < row_ptr[ref + 1]; ++i)
      c += jxo_found(ind, row_ptr[cur], row_ptr[cur + 1] - 1, ind[i]);
    cnt[j - base] = c;
  }
}

/*
 * FP64 oracle: the same Jaccard definition evaluated in double precision with exact-order
 * independence for practical purposes (S and I accumulated in double):
 *   S[v] = sum of w over N(v) (or deg), I = sum of w over N(u) n N(v) (or count),
 *   J = I / (S[u] + S[v] - I).
 * Used to report the error of both the reference order and the engine.
 */
void jxo_jaccard_f64_rows(int32_t n, const int32_t *row_ptr, const int32_t *ind, const float *w,
                          int32_t r0, int32_t r1, double *out, int nthreads) {
  jxo_threads(nthreads);
  double *S = (double *)malloc(sizeof(double) * (n > 0 ? n : 1));
  if (!S) return;
#pragma omp parallel for schedule(dynamic, 256)
  for (int32_t v = 0; v < n; ++v) {
    double s = 0.0;
    for (int32_t k = row_ptr[v]; k < row_ptr[v + 1]; ++k) s += w ? (double)w[ind[k]] : 1.0;
    S[v] = s;
  }
  const int64_t base = row_ptr[r0];
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t j = base; j < (int64_t)row_ptr[r1]; ++j) {
    const int32_t row = jxo_row_of(row_ptr, r0, r1, j);
    const int32_t col = ind[j];
    const int32_t Ni = row_ptr[row + 1] - row_ptr[row];
    const int32_t Nj = row_ptr[col + 1] - row_ptr[col];
    const int32_t ref = (Ni < Nj) ? row : col;
    const int32_t cur = (Ni < Nj) ? col : row;
    double I = 0.0;
    for (int32_t i = row_ptr[ref]; i < row_ptr[ref + 1]; ++i)
      if (jxo_found(ind, row_ptr[cur], row_ptr[cur + 1] - 1, ind[i]))
        I += w ? (double)w[ind[i]] : 1.0;
    out[j - base] = I / (S[row] + S[col] - I);
  }
  free(S);
}

/*
 * jaccard_list restated with its intended semantics (standalone_algorithms.hpp:109-133,
 * jaccard.cpp:957-988; the reference's pair kernel writes weight_i[i] instead of
 * weight_i[idx], jaccard.cpp:517, 528): each pair (first, second) is computed like the
 * vertex-centric edge (first, second) -- ref = shorter list, ties to second
 * (jaccard.cpp:476-477), sum in the 8-i-lane order, J = I / (S_first + S_second - I).
 */
void jxo_jaccard_list(int32_t n, const int32_t *row_ptr, const int32_t *ind, const float *w,
                      int64_t np, const int32_t *first, const int32_t *second, float *out,
                      int nthreads) {
  jxo_threads(nthreads);
  float *S = (float *)malloc(sizeof(float) * (n > 0 ? n : 1));
  if (!S) return;
  jxo_rowsum(n, row_ptr, ind, w, S, nthreads);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t p = 0; p < np; ++p) {
    const int32_t row = first[p], col = second[p];
    const int32_t Ni = row_ptr[row + 1] - row_ptr[row];
    const int32_t Nj = row_ptr[col + 1] - row_ptr[col];
    const int32_t ref = (Ni < Nj) ? row : col;
    const int32_t cur = (Ni < Nj) ? col : row;
    float acc = 0.0f;
    for (int il = 0; il < JXO_IS_I_LANES; ++il)
      for (int32_t i = row_ptr[ref] + il; i < row_ptr[ref + 1]; i += JXO_IS_I_LANES) {
        const int32_t ref_col = ind[i];
        const float ref_val = w ? w[ref_col] : 1.0f;
        if (jxo_found(ind, row_ptr[cur], row_ptr[cur + 1] - 1, ref_col)) acc = ref_val + acc;
      }
    const float Ws = S[row] + S[col];
    out[p] = acc / (Ws - acc);
  }
  free(S);
}

/*
 * Cost proxy of the reference's IS kernel per row (used to extrapolate a timed sample of the
 * reference's work-groups to the whole call): work[row] = sum over the row's edges of
 * min(d_u, d_v) * (1 + log2(max(d_u, d_v))), the binary searches of the shorter list
 * (jaccard.cpp:333-367).
 */
void jxo_row_work(int32_t n, const int32_t *row_ptr, const int32_t *ind, double *work, int nthreads) {
  jxo_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int32_t row = 0; row < n; ++row) {
    const int32_t du = row_ptr[row + 1] - row_ptr[row];
    double s = 0.0;
    for (int32_t j = row_ptr[row]; j < row_ptr[row + 1]; ++j) {
      const int32_t v = ind[j];
      const int32_t dv = row_ptr[v + 1] - row_ptr[v];
      const int32_t mn = du < dv ? du : dv, mx = du < dv ? dv : du;
      s += (double)mn * (1.0 + log2((double)(mx > 1 ? mx : 1)));
    }
    work[row] = s;
  }
}

/*
 * Cost proxy per work-group of the reference's dominant kernel, for timing samples that run
 * every K-th work-group.  Vertex-centric (ec == 0): Jaccard_IsKernel's group g of G =
 * min(ceil(n / 8), 65535) holds rows 8g .. 8g+7, then every 8G rows further (jaccard.cpp:413-417
 * and its row grid-stride); edge-centric: Jaccard_ec_unweighted's group g of G =
 * min(ceil(e / 256), 65535) holds edges 256g .. 256g+255, then every 256G edges further
 * (jaccard.cpp:750-753).  out[g] = sum over the group's edges of
 * min(d_u, d_v) * (1 + log2(max(d_u, d_v))).  Returns G.
 */
int64_t jxo_group_work(int ec, int32_t n, const int32_t *row_ptr, const int32_t *ind, double *out,
                       int nthreads) {
  jxo_threads(nthreads);
  const int64_t e = row_ptr[n];
  const int64_t span = ec ? 256 : 8;
  const int64_t units = ec ? e : n;
  int64_t G = (units + span - 1) / span;
  if (G > 65535) G = 65535;
  if (G < 1) G = 1;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t g = 0; g < G; ++g) {
    double s = 0.0;
    for (int64_t base = g * span; base < units; base += span * G)
      for (int64_t x = base; x < base + span && x < units; ++x) {
        int64_t j0, j1;
        int32_t row;
        if (ec) { /* edge x: its row by binary search */
          int32_t lo = 0, hi = n - 1;
          while (lo < hi) {
            const int32_t mid = lo + (hi - lo + 1) / 2;
            if ((int64_t)row_ptr[mid] <= x) lo = mid; else hi = mid - 1;
          }
          row = lo;
          j0 = x;
          j1 = x + 1;
        } else {
          row = (int32_t)x;
          j0 = row_ptr[row];
          j1 = row_ptr[row + 1];
        }
        const int32_t du = row_ptr[row + 1] - row_ptr[row];
        for (int64_t j = j0; j < j1; ++j) {
          const int32_t v = ind[j];
          const int32_t dv = row_ptr[v + 1] - row_ptr[v];
          const int32_t mn = du < dv ? du : dv, mx = du < dv ? dv : du;
          s += (double)mn * (1.0 + log2((double)(mx > 1 ? mx : 1)));
        }
      }
    out[g] = s;
  }
  return G;
}
