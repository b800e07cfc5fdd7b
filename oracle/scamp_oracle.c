/*
 * scamp_oracle.c -- CPU oracle for the SCAMP matrix-profile join.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU engine is
 * compared against: only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference legs of bench.py load it.  The engine (libscamp_gb300.so) never
 * links it and has no CPU fallback.
 *
 * It restates the reference's CPU algorithm (zpzim/GPU-SCRIMP-LARGE, files cited
 * per function below) in plain C, with two deliberate differences that make it
 * a stricter checker:
 *   1. Correlations are kept in double end to end (the reference rounds r to
 *      float32 before comparing, src/cpu_kernels.cpp:146-149, 267-270), so the
 *      oracle can also check FP64 results to 1e-9.  The packed float32/uint32
 *      profile (src/common.h:70-74) is produced from the double result.
 *   2. The whole join is one tile: every diagonal is seeded once at row 0 and
 *      advanced with the exact recurrence over its full length (the reference
 *      re-seeds at each max_tile_size boundary, src/SCAMP.cpp:25-90).
 *      Ties between equal double correlations go to the smallest index.
 *
 * Parity pins: tests/test_oracle_pin.py checks this file against the golden
 * outputs shipped with the reference (test/SampleOutput/mp_*, mpi_*) and
 * against the reference's own CPU path compiled from its sources
 * (oracle/Makefile -> oracle/_ref/).
 *
 * Build: cc -O3 -fopenmp -fPIC -shared scamp_oracle.c -o liboracle.so -lm
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_PROFILE_1NN_INDEX 1
#define ORACLE_PROFILE_SUM_THRESH 2

/* src/cpu_stats.cpp:4 */
static const double FLATNESS_EPSILON = 1e-13;

/* Restates convert_non_finite_to_zero, src/cpu_stats.cpp:11-29: non-finite
 * samples become 0 and nanwin[i] marks every window that held one. */
void oracle_clean(const double *T, int64_t n, int64_t m, double *T_clean,
                  unsigned char *nanwin) {
  int64_t since = m;
  for (int64_t i = 0; i < n; ++i) {
    if (isfinite(T[i])) {
      T_clean[i] = T[i];
    } else {
      since = 0;
      T_clean[i] = 0;
    }
    if (i >= m - 1) nanwin[i - m + 1] = since < m;
    since++;
  }
}

/* Restates moving_mean, src/cpu_stats.cpp:50-75: rolling window sum with a
 * TwoSum error term (Ogita et al.), divided by m. */
static void moving_mean(const double *a, int64_t n, int64_t w, double *out) {
  double p = a[0], s = 0;
  for (int64_t i = 1; i < w; ++i) {
    double x = p + a[i];
    double z = x - p;
    s += (p - (x - z)) + (a[i] - z);
    p = x;
  }
  out[0] = (p + s) / w;
  for (int64_t i = w; i < n; ++i) {
    double x = p - a[i - w];
    double z = x - p;
    s += (p - (x - z)) - (a[i - w] + z);
    p = x;
    x = p + a[i];
    z = x - p;
    s += (p - (x - z)) + (a[i] - z);
    p = x;
    out[i - w + 1] = (p + s) / w;
  }
}

/* Restates fast_sum_of_squared_difference, src/cpu_stats.cpp:103-120. */
static void fast_ssd(const double *a, int64_t n, const double *mu, int64_t w,
                     double *out) {
  double sum = 0;
  for (int64_t i = 0; i < w; ++i) {
    double v = a[i] - mu[0];
    sum += v * v;
  }
  out[0] = sum;
  for (int64_t i = 1; i < n - w + 1; ++i) {
    out[i] = out[i - 1] + ((a[i - 1] - mu[i - 1]) + (a[i + w - 1] - mu[i])) *
                              (a[i + w - 1] - a[i - 1]);
  }
}

/* Brute-force O(nm) forms, src/cpu_stats.cpp:31-41 and :85-97 (ULTRA). */
static void brute_mean(const double *a, int64_t n, int64_t w, double *out) {
  for (int64_t i = 0; i + w <= n; ++i) {
    double s = 0;
    for (int64_t j = 0; j < w; ++j) s += a[i + j];
    out[i] = s / w;
  }
}
static void brute_ssd(const double *a, int64_t n, const double *mu, int64_t w,
                      double *out) {
  for (int64_t i = 0; i + w <= n; ++i) {
    double s = 0;
    for (int64_t j = 0; j < w; ++j) {
      double v = a[i + j] - mu[i];
      s += v * v;
    }
    out[i] = s;
  }
}

/* Restates compute_statistics_cpu, src/cpu_stats.cpp:123-160.
 * T_clean must already be cleaned (oracle_clean).  Outputs have n-m+1
 * entries; norms[] holds the inverse norm 1/sqrt(ssd), NaN for windows that
 * held a non-finite sample or whose ssd <= 1e-13; df/dg are 0 at the last
 * window. */
void oracle_stats(const double *T_clean, const unsigned char *nanwin, int64_t n,
                  int64_t m, int high_precision, double *means, double *norms,
                  double *df, double *dg) {
  int64_t ns = n - m + 1;
  if (high_precision) {
    brute_mean(T_clean, n, m, means);
    brute_ssd(T_clean, n, means, m, norms);
  } else {
    moving_mean(T_clean, n, m, means);
    fast_ssd(T_clean, n, means, m, norms);
  }
  for (int64_t i = 0; i < ns; ++i) {
    if (nanwin[i]) {
      norms[i] = NAN;
    } else if (norms[i] <= FLATNESS_EPSILON) {
      norms[i] = NAN;
    } else {
      norms[i] = 1.0 / sqrt(norms[i]);
    }
  }
  for (int64_t i = 0; i < ns - 1; ++i) {
    df[i] = (T_clean[i + m] - T_clean[i]) / 2.0;
    dg[i] = (T_clean[i + m] - means[i + 1]) + (T_clean[i] - means[i]);
  }
  df[ns - 1] = 0;
  dg[ns - 1] = 0;
}

/* Restates compute_combined_stats_cpu, src/cpu_stats.cpp:162-196: the
 * update terms ULTRA uses instead of df/dg (src/tile.cpp:404-409).  Series A
 * (role 0) gets df = -(T[i] - mu[i]), dg = T[i+m] - mu[i+1]; series B (role 1)
 * gets df = T[i+m] - mu'[i+1], dg = T[i] - mu'[i+1], with mu' the brute-force
 * (m-1)-sample means.  The reference fills the last window's terms from one
 * sample past the series; the recurrence never uses them, and they are 0
 * here. */
void oracle_combined_terms(const double *T_clean, int64_t n, int64_t m,
                           const double *means, int role, double *df,
                           double *dg) {
  int64_t ns = n - m + 1;
  for (int64_t i = 0; i < ns - 1; ++i) {
    if (role == 0) {
      df[i] = -1 * (T_clean[i] - means[i]);
      dg[i] = T_clean[i + m] - means[i + 1];
    } else {
      double sum = 0;
      for (int64_t j = 0; j < m - 1; ++j) sum += T_clean[i + 1 + j];
      double mu1 = sum / (double)(m - 1);
      df[i] = T_clean[i + m] - mu1;
      dg[i] = T_clean[i] - mu1;
    }
  }
  df[ns - 1] = 0;
  dg[ns - 1] = 0;
}

/* Restates compute_QT_CPU, src/qt_helper.cpp:52-72: the first row of a tile,
 * QT[j] = sum_t (T[j+t] - mu_T[j]) * (Q[t] - mu_Q[0]), with window means from
 * a plain rolling sum, for j in [0, count). */
void oracle_qt_row(const double *T, const double *Q, int64_t count, int64_t m,
                   double *QT) {
  double rolling = 0, qmean = 0;
  for (int64_t i = 0; i < m; ++i) {
    rolling += T[i];
    qmean += Q[i];
  }
  qmean /= m;
  for (int64_t i = 0; i < count; ++i) {
    double mu = rolling / m;
    double s = 0;
    for (int64_t j = 0; j < m; ++j) s += (T[i + j] - mu) * (Q[j] - qmean);
    QT[i] = s;
    rolling = rolling - T[i] + T[i + m];
  }
}

/* Seed for diagonal d of a (rows=R, cols=C) band problem: cov of row window 0
 * and column window d, each centred by its own (compensated) window mean. */
static double seed_cov(const double *Rs, const double *Cs, const double *mu_r,
                       const double *mu_c, int64_t d, int64_t m) {
  double s = 0, comp = 0;
  for (int64_t t = 0; t < m; ++t) {
    double p = (Cs[d + t] - mu_c[d]) * (Rs[t] - mu_r[0]);
    /* Neumaier summation */
    double x = s + p;
    if (fabs(s) >= fabs(p))
      comp += (s - x) + p;
    else
      comp += (p - x) + s;
    s = x;
  }
  return s + comp;
}

typedef struct {
  const double *a;
  int64_t na;
  const double *b; /* NULL for a self-join */
  int64_t nb;
  int64_t m;
  int profile_type; /* 1 = 1NN_INDEX, 2 = SUM_THRESH */
  int computing_rows;
  int computing_cols;
  int keep_rows_separate;
  int is_aligned;
  int64_t start_row; /* distributed_start_row, -1 if unused */
  int64_t start_col; /* distributed_start_col, -1 if unused */
  double threshold;
  int threads;      /* 0 = all available */
  int brute_force;  /* 1: every cell from a fresh compensated dot product */
  int high_precision_stats; /* 1: ULTRA-style brute force means / ssd */
  int exact_flat; /* 1: decide flatness (ssd <= 1e-13) from an exact ssd */
  int combined_terms; /* 1: ULTRA's combined update terms (see below) */
} oracle_args;

typedef struct {
  /* Per window of A (columns). Either may be NULL. */
  double *corr_a;   /* 1NN_INDEX: best correlation (double), -2 if none */
  int64_t *idx_a;   /* 1NN_INDEX: index of best, -1 if none */
  double *sum_a;    /* SUM_THRESH */
  /* Per window of B (rows), used when keep_rows_separate. */
  double *corr_b;
  int64_t *idx_b;
  double *sum_b;
} oracle_out;

/* Per-thread partial profile. */
typedef struct {
  double *best;
  int64_t *idx;
  double *sum;
} partial_t;

static inline void upd_max(partial_t *p, int64_t k, double r, int64_t other) {
  /* strict '>' keeps NaN out (src/cpu_kernels.cpp:51); equal values go to
   * the smaller index so the result does not depend on thread count. */
  if (r > p->best[k] || (r == p->best[k] && other < p->idx[k])) {
    p->best[k] = r;
    p->idx[k] = other;
  }
}

typedef struct {
  /* row series (windows i) and column series (windows j) */
  const double *Tr, *Tc;
  const double *mu_r, *mu_c, *in_r, *in_c, *df_r, *df_c, *dg_r, *dg_c;
  int64_t n_r, n_c; /* window counts */
  int64_t d_lo, d_hi; /* diagonal range [d_lo, d_hi) */
  int64_t x_lo, x_hi; /* excluded diagonals [x_lo, x_hi) (empty if x_lo>=x_hi) */
  int col_target;     /* 0 -> A partial, 1 -> B partial, -1 none */
  int row_target;
} band_t;

/* Brute-force correlation of row window i and column window j, with the
 * reference's NaN / flatness rule taken from the inverse norms. */
static double brute_corr(const band_t *bd, int64_t i, int64_t j, int64_t m) {
  if (isnan(bd->in_r[i]) || isnan(bd->in_c[j])) return NAN;
  double s = 0, comp = 0, sr = 0, cr = 0, sc = 0, cc = 0;
  for (int64_t t = 0; t < m; ++t) {
    double x = bd->Tr[i + t] - bd->mu_r[i];
    double y = bd->Tc[j + t] - bd->mu_c[j];
    double terms[3] = {x * y, x * x, y * y};
    double *acc[3] = {&s, &sr, &sc};
    double *cmp[3] = {&comp, &cr, &cc};
    for (int q = 0; q < 3; ++q) {
      double a0 = *acc[q], p = terms[q], z = a0 + p;
      if (fabs(a0) >= fabs(p))
        *cmp[q] += (a0 - z) + p;
      else
        *cmp[q] += (p - z) + a0;
      *acc[q] = z;
    }
  }
  return (s + comp) / sqrt((sr + cr) * (sc + cc));
}

#define STRIP 256

/* One strip of STRIP diagonals of a band problem.  Restates the CPU do_tile
 * loop (src/cpu_kernels.cpp:117-199): r = cov * invnorm_col * invnorm_row,
 * reduce per column and per row, then advance every diagonal with
 * cov += df_col*dg_row + df_row*dg_col (src/cpu_kernels.cpp:166-171). */
static void do_strip(const band_t *bd, int64_t d0, int64_t d1, int64_t m,
                     int ptype, double thr, int brute, partial_t *pc,
                     partial_t *pr) {
  double cov[STRIP];
  double r[STRIP];
  int64_t nd = d1 - d0;
  for (int64_t s = 0; s < nd; ++s)
    cov[s] = brute ? 0 : seed_cov(bd->Tr, bd->Tc, bd->mu_r, bd->mu_c, d0 + s, m);
  int64_t rows = bd->n_c - d0;
  if (rows > bd->n_r) rows = bd->n_r;
  int64_t i = 0;
  /* Full-width rows of a strip clear of the excluded diagonals: the same
   * arithmetic in loops of constant length, which the compiler vectorises
   * (the reference's unrolled fast case, src/cpu_kernels.cpp:139-172). */
  if (!brute && nd == STRIP && !(bd->x_lo < d1 && bd->x_hi > d0)) {
    int64_t fast = bd->n_c - d1 + 1; /* rows where every diagonal is inside */
    if (fast > rows) fast = rows;
    for (; i < fast; ++i) {
      const double ir = bd->in_r[i];
      const double *inc = bd->in_c + i + d0;
      const double *dfc = bd->df_c + i + d0;
      const double *dgc = bd->dg_c + i + d0;
      for (int s = 0; s < STRIP; ++s) r[s] = cov[s] * inc[s] * ir;
      if (ptype == ORACLE_PROFILE_1NN_INDEX) {
        if (pc)
          for (int s = 0; s < STRIP; ++s) upd_max(pc, i + d0 + s, r[s], i);
        if (pr) {
          double best = -2;
          int64_t bj = -1;
          for (int s = 0; s < STRIP; ++s)
            if (r[s] > best) {
              best = r[s];
              bj = i + d0 + s;
            }
          if (bj >= 0) upd_max(pr, i, best, bj);
        }
      } else {
        if (pc)
          for (int s = 0; s < STRIP; ++s)
            if (r[s] > thr) pc->sum[i + d0 + s] += r[s];
        if (pr) {
          double acc = 0;
          for (int s = 0; s < STRIP; ++s)
            if (r[s] > thr) acc += r[s];
          pr->sum[i] += acc;
        }
      }
      const double dfr = bd->df_r[i], dgr = bd->dg_r[i];
      for (int s = 0; s < STRIP; ++s) {
        cov[s] += dfc[s] * dgr;
        cov[s] += dfr * dgc[s];
      }
    }
  }
  for (; i < rows; ++i) {
    int64_t lim = bd->n_c - i - d0; /* diagonals still inside the matrix */
    if (lim > nd) lim = nd;
    double ir = bd->in_r[i];
    for (int64_t s = 0; s < lim; ++s) {
      int64_t d = d0 + s;
      int64_t j = i + d;
      double v = brute ? brute_corr(bd, i, j, m) : cov[s] * bd->in_c[j] * ir;
      if (d >= bd->x_lo && d < bd->x_hi) v = NAN;
      r[s] = v;
    }
    if (ptype == ORACLE_PROFILE_1NN_INDEX) {
      if (pc)
        for (int64_t s = 0; s < lim; ++s) upd_max(pc, i + d0 + s, r[s], i);
      if (pr) {
        double best = -2;
        int64_t bj = -1;
        for (int64_t s = 0; s < lim; ++s)
          if (r[s] > best) {
            best = r[s];
            bj = i + d0 + s;
          }
        if (bj >= 0) upd_max(pr, i, best, bj);
      }
    } else {
      if (pc)
        for (int64_t s = 0; s < lim; ++s)
          if (r[s] > thr) pc->sum[i + d0 + s] += r[s];
      if (pr) {
        double acc = 0;
        for (int64_t s = 0; s < lim; ++s)
          if (r[s] > thr) acc += r[s];
        pr->sum[i] += acc;
      }
    }
    if (!brute) {
      double dfr = bd->df_r[i], dgr = bd->dg_r[i];
      for (int64_t s = 0; s < lim; ++s) {
        int64_t j = i + d0 + s;
        cov[s] += bd->df_c[j] * dgr;
        cov[s] += dfr * bd->dg_c[j];
      }
    }
  }
}

typedef struct {
  double *T_clean;
  unsigned char *nanwin;
  double *mu, *in, *df, *dg;
  double *df_rows, *dg_rows; /* the row role's terms (ULTRA self-join), or df/dg */
  int64_t n, ns;
} series_t;

static int series_init(series_t *s, const double *T, int64_t n, int64_t m,
                       int hp, int exact_flat, int role, int rows_role) {
  s->n = n;
  s->ns = n - m + 1;
  s->T_clean = malloc(sizeof(double) * n);
  s->nanwin = malloc(s->ns);
  s->mu = malloc(sizeof(double) * s->ns);
  s->in = malloc(sizeof(double) * s->ns);
  s->df = malloc(sizeof(double) * s->ns);
  s->dg = malloc(sizeof(double) * s->ns);
  if (!s->T_clean || !s->nanwin || !s->mu || !s->in || !s->df || !s->dg)
    return -1;
  oracle_clean(T, n, m, s->T_clean, s->nanwin);
  oracle_stats(s->T_clean, s->nanwin, n, m, hp, s->mu, s->in, s->df, s->dg);
  s->df_rows = s->df;
  s->dg_rows = s->dg;
  /* ULTRA (role >= 0): this series' combined terms replace df/dg; a
   * self-join's rows (rows_role >= 0) take the other role's terms */
  if (role >= 0)
    oracle_combined_terms(s->T_clean, n, m, s->mu, role, s->df, s->dg);
  if (rows_role >= 0 && rows_role != role) {
    s->df_rows = malloc(sizeof(double) * s->ns);
    s->dg_rows = malloc(sizeof(double) * s->ns);
    if (!s->df_rows || !s->dg_rows) return -1;
    oracle_combined_terms(s->T_clean, n, m, s->mu, rows_role, s->df_rows,
                          s->dg_rows);
  }
  if (exact_flat) {
    /* The reference's sequential ssd recurrence can leave a rounding residue
     * above 1e-13 on exactly flat windows; this mode applies the flatness
     * rule to a directly summed ssd instead. */
    for (int64_t i = 0; i < s->ns; ++i) {
      if (s->nanwin[i]) continue;
      double mu = 0;
      for (int64_t t = 0; t < m; ++t) mu += s->T_clean[i + t];
      mu /= m;
      double ss = 0;
      for (int64_t t = 0; t < m; ++t) {
        double v = s->T_clean[i + t] - mu;
        ss += v * v;
      }
      s->in[i] = ss <= FLATNESS_EPSILON ? NAN : 1.0 / sqrt(ss);
    }
  }
  return 0;
}

static void series_free(series_t *s) {
  if (s->df_rows != s->df) free(s->df_rows);
  if (s->dg_rows != s->dg) free(s->dg_rows);
  free(s->T_clean);
  free(s->nanwin);
  free(s->mu);
  free(s->in);
  free(s->df);
  free(s->dg);
}

static band_t make_band(const series_t *rows, const series_t *cols,
                        int64_t d_lo, int64_t d_hi, int col_target,
                        int row_target) {
  band_t b;
  b.Tr = rows->T_clean;
  b.Tc = cols->T_clean;
  b.mu_r = rows->mu;
  b.mu_c = cols->mu;
  b.in_r = rows->in;
  b.in_c = cols->in;
  b.df_r = rows->df_rows;
  b.df_c = cols->df;
  b.dg_r = rows->dg_rows;
  b.dg_c = cols->dg;
  b.n_r = rows->ns;
  b.n_c = cols->ns;
  b.d_lo = d_lo;
  b.d_hi = d_hi;
  b.x_lo = 0;
  b.x_hi = 0;
  b.col_target = col_target;
  b.row_target = row_target;
  return b;
}

/* Full join.  Cell geometry follows the reference:
 *  - self-join: upper triangle, diagonals d >= m/4 (src/tile.cpp:12-38);
 *    column results and row results both land in profile A unless
 *    keep_rows_separate (src/tile.cpp:532-541);
 *  - AB-join: every (row window of B, column window of A); the part below the
 *    main diagonal runs transposed (src/tile.cpp:645-707,
 *    src/cpu_kernels.cpp:306-311); is_aligned excludes |i-j| < m/4 measured in
 *    global positions (src/tile.cpp:44-138); A's profile is updated iff
 *    computing_cols, B's iff computing_rows && keep_rows_separate.
 * Returns 0 on success. */
int oracle_join(const oracle_args *args, oracle_out *out) {
  int64_t m = args->m;
  if (m < 3 || args->na < m) return -1;
  int self = args->b == NULL;
  if (!self && args->nb < m) return -1;
  int ptype = args->profile_type;
  if (ptype != ORACLE_PROFILE_1NN_INDEX && ptype != ORACLE_PROFILE_SUM_THRESH)
    return -2;
  series_t A, B;
  /* ULTRA: A takes the "A" terms and B the "B" terms (the reference's
   * roles); a self-join's rows take the "B" terms of A */
  int ct = args->combined_terms;
  if (series_init(&A, args->a, args->na, m, args->high_precision_stats,
                  args->exact_flat, ct ? 0 : -1, (ct && self) ? 1 : -1))
    return -3;
  if (!self && series_init(&B, args->b, args->nb, m, args->high_precision_stats,
                           args->exact_flat, ct ? 1 : -1, -1)) {
    series_free(&A);
    return -3;
  }
  const series_t *Bp = self ? &A : &B;
  int64_t nsa = A.ns, nsb = Bp->ns;
  int64_t excl = m / 4;

  /* target 0 = A's profile, 1 = B's profile, -1 = not computed */
  int tgt_cols_A = args->computing_cols ? 0 : -1;
  int tgt_rows_B;
  if (self) {
    tgt_rows_B = args->computing_rows ? (args->keep_rows_separate ? 1 : 0) : -1;
  } else {
    tgt_rows_B = (args->computing_rows && args->keep_rows_separate) ? 1 : -1;
  }

  band_t bands[2];
  int nbands = 0;
  if (self) {
    bands[nbands++] = make_band(&A, &A, excl, nsa, tgt_cols_A, tgt_rows_B);
  } else {
    /* upper part: rows = B, cols = A, d = j - i >= 0 */
    bands[nbands] = make_band(Bp, &A, 0, nsa, tgt_cols_A, tgt_rows_B);
    /* lower part transposed: rows = A, cols = B, d = i_B - j_A >= 1 */
    bands[nbands + 1] = make_band(&A, Bp, 1, nsb, tgt_rows_B, tgt_cols_A);
    if (args->is_aligned) {
      int64_t off = 0; /* global col - global row offset of window (0,0) */
      if (args->start_row >= 0 && args->start_col >= 0)
        off = args->start_col - args->start_row;
      /* upper: excluded when |d + off| < excl */
      bands[nbands].x_lo = -off - excl + 1;
      bands[nbands].x_hi = -off + excl;
      /* lower: original d = -d', excluded when |off - d'| < excl */
      bands[nbands + 1].x_lo = off - excl + 1;
      bands[nbands + 1].x_hi = off + excl;
    }
    nbands += 2;
  }

  int nth = args->threads;
#ifdef _OPENMP
  if (nth <= 0) nth = omp_get_max_threads();
#else
  nth = 1;
#endif
  int64_t nsmax = nsa > nsb ? nsa : nsb;
  partial_t *parts = calloc((size_t)nth * 2, sizeof(partial_t));
  int used[2] = {0, 0};
  for (int bi = 0; bi < nbands; ++bi) {
    if (bands[bi].col_target >= 0) used[bands[bi].col_target] = 1;
    if (bands[bi].row_target >= 0) used[bands[bi].row_target] = 1;
  }
  for (int t = 0; t < nth * 2; ++t) {
    if (!used[t % 2]) continue;
    if (ptype == ORACLE_PROFILE_1NN_INDEX) {
      parts[t].best = malloc(sizeof(double) * nsmax);
      parts[t].idx = malloc(sizeof(int64_t) * nsmax);
      for (int64_t k = 0; k < nsmax; ++k) {
        parts[t].best[k] = -2;
        parts[t].idx[k] = -1;
      }
    } else {
      parts[t].sum = calloc(nsmax, sizeof(double));
    }
  }

  for (int bi = 0; bi < nbands; ++bi) {
    band_t *bd = &bands[bi];
    int64_t nstrips = (bd->d_hi - bd->d_lo + STRIP - 1) / STRIP;
    if (bd->d_hi <= bd->d_lo) continue;
    if (bd->col_target < 0 && bd->row_target < 0) continue;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
    for (int64_t st = 0; st < nstrips; ++st) {
      int t = 0;
#ifdef _OPENMP
      t = omp_get_thread_num();
#endif
      int64_t d0 = bd->d_lo + st * STRIP;
      int64_t d1 = d0 + STRIP;
      if (d1 > bd->d_hi) d1 = bd->d_hi;
      partial_t *pc = bd->col_target >= 0 ? &parts[t * 2 + bd->col_target] : NULL;
      partial_t *pr = bd->row_target >= 0 ? &parts[t * 2 + bd->row_target] : NULL;
      do_strip(bd, d0, d1, m, ptype, args->threshold, args->brute_force, pc, pr);
    }
  }

  /* merge the per-thread partials */
  for (int which = 0; which < 2; ++which) {
    int64_t ns = which == 0 ? nsa : nsb;
    double *corr = which == 0 ? out->corr_a : out->corr_b;
    int64_t *idx = which == 0 ? out->idx_a : out->idx_b;
    double *sum = which == 0 ? out->sum_a : out->sum_b;
    for (int64_t k = 0; k < ns; ++k) {
      double best = -2, s = 0;
      int64_t bi = -1;
      for (int t = 0; t < nth && used[which]; ++t) {
        partial_t *p = &parts[t * 2 + which];
        if (p->best && (p->best[k] > best ||
                        (p->best[k] == best && p->idx[k] >= 0 &&
                         (bi < 0 || p->idx[k] < bi)))) {
          best = p->best[k];
          bi = p->idx[k];
        }
        if (p->sum) s += p->sum[k];
      }
      if (corr) corr[k] = best;
      if (idx) idx[k] = bi;
      if (sum) sum[k] = s;
    }
  }

  for (int t = 0; t < nth * 2; ++t) {
    free(parts[t].best);
    free(parts[t].idx);
    free(parts[t].sum);
  }
  free(parts);
  series_free(&A);
  if (!self) series_free(&B);
  return 0;
}

/* Packs a double correlation and index into the reference's 1NN_INDEX entry
 * (src/common.h:70-74: float corr in the low word, uint32 index in the high
 * word); no match is {-2.0f, 0xFFFFFFFF} (src/common.cpp:294-299). */
void oracle_pack(const double *corr, const int64_t *idx, int64_t n,
                 uint64_t *packed) {
  for (int64_t k = 0; k < n; ++k) {
    float f = idx[k] < 0 ? -2.0f : (float)corr[k];
    uint32_t fb;
    memcpy(&fb, &f, 4);
    uint32_t ib = idx[k] < 0 ? 0xFFFFFFFFu : (uint32_t)idx[k];
    packed[k] = ((uint64_t)ib << 32) | fb;
  }
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
