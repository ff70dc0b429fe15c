/*
 * oracle.c — CPU restatement of skylens-stream-rs's descriptor-matching path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the parity checker and the timed CPU
 * baseline ("port"); the product library never links, loads or calls it.
 *
 * Every function restates one piece of the reference (Rust, CPU only):
 *   orc_lcg_next / orc_lcg_gauss   crates/core/src/matching.rs:1140-1153 (test Lcg)
 *   orc_feature                    crates/core/src/matching.rs:1580-1596 (test `feature`)
 *   orc_match_fixture              crates/core/src/matching.rs:1638-1656 (`match_fixture`)
 *   orc_sq_dist                    crates/core/src/matching.rs:144-155 (`sq_dist`, spec at :2345-2357)
 *   orc_sq_dist_seq                crates/core/src/matching.rs:2373-2377 (sequential fold, boundary test)
 *   orc_ratio_match                crates/core/src/matching.rs:157-215 (`ratio_match`, MATCH_BLOCK = 64)
 *   orc_ratio_match_naive          crates/core/src/matching.rs:1597-1636 (`ratio_match_reference`)
 *   orc_pairs_hash                 crates/core/src/matching.rs:1866-1878 (`pairs_hash`, FNV-1a 64)
 *   orc_candidate_pairs            crates/core/src/matching.rs:14-40
 *   orc_scheduled_pairs            crates/core/src/matching.rs:103-142
 *   orc_sampson_residual           crates/core/src/two_view.rs:456-465 (`sampson_residual`)
 *   orc_sampson_score              crates/core/src/two_view.rs:804-823 (`inliers_of`,
 *                                  `count_at_least` of ransac_essential_inner), batched
 * plus orc_sq_dist_f64, an FP64 distance used only to report the error of
 * low-precision distances (never for a match decision).
 *
 * Floating point: build with -O3 -ffp-contract=off (no FMA contraction, as in
 * Rust). Every f32 operation below is one IEEE round-to-nearest operation in
 * the same order as the reference. The f64 ln/cos of Lcg::gauss come from the
 * platform libm, as Rust's f64::ln/cos do.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define DESC_LEN 128
#define MATCH_BLOCK 64

/* ---------------------------------------------------------------- Lcg */

/* matching.rs:1141-1148: state = state*6364136223846793005 + 1442695040888963407
 * (wrapping); returns (state >> 11) / 2^53. */
double orc_lcg_next(uint64_t *s) {
    *s = *s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(*s >> 11) / (double)(1ULL << 53);
}

/* matching.rs:1149-1152: Box-Muller, u1 clamped to >= 1e-300. */
double orc_lcg_gauss(uint64_t *s) {
    double u1 = orc_lcg_next(s);
    if (!(u1 >= 1e-300)) u1 = 1e-300; /* f64::max(u1, 1e-300); u1 is never NaN */
    double u2 = orc_lcg_next(s);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* matching.rs:1580-1596: 128 uniform draws cast to f32, divided by the f32
 * L2 norm (sum of squares in index order, then sqrt). */
void orc_feature(uint64_t *s, float *out) {
    for (int k = 0; k < DESC_LEN; k++) out[k] = (float)orc_lcg_next(s);
    float acc = -0.0f;
    for (int k = 0; k < DESC_LEN; k++) {
        float sq = out[k] * out[k];
        acc = acc + sq;
    }
    float n = sqrtf(acc);
    for (int k = 0; k < DESC_LEN; k++) out[k] = out[k] / n;
}

/* h[k] += scale * (f32)gauss(), component order (matching.rs:1649-1651, 1717-1719). */
void orc_perturb(uint64_t *s, float *h, float scale) {
    for (int k = 0; k < DESC_LEN; k++) {
        float g = (float)orc_lcg_gauss(s);
        float add = scale * g;
        h[k] = h[k] + add;
    }
}

/* Number of b rows match_fixture makes before the `extra` fresh draws. */
int64_t orc_match_fixture_copies(int64_t na) {
    int64_t m = 0;
    for (int64_t i = 0; i < na; i++) {
        if (i % 3 == 2) continue;
        m += 1 + (i % 7 == 0);
    }
    return m;
}

/* matching.rs:1638-1656. a: na x 128, b: (copies(na) + extra) x 128. */
void orc_match_fixture(uint64_t seed, int64_t na, int64_t extra, float *a, float *b) {
    uint64_t s = seed;
    for (int64_t i = 0; i < na; i++) orc_feature(&s, a + i * DESC_LEN);
    int64_t m = 0;
    for (int64_t i = 0; i < na; i++) {
        if (i % 3 == 2) continue;
        int reps = 1 + (i % 7 == 0);
        for (int r = 0; r < reps; r++) {
            float *h = b + m * DESC_LEN;
            memcpy(h, a + i * DESC_LEN, sizeof(float) * DESC_LEN);
            orc_perturb(&s, h, 0.03f);
            m++;
        }
    }
    for (int64_t e = 0; e < extra; e++) orc_feature(&s, b + (m + e) * DESC_LEN);
}

/* ----------------------------------------------------------- distances */

/* matching.rs:144-155 / spec :2345-2357. Component 8c+k accumulates into lane k
 * (t = p - r; acc[k] += t*t, c = 0..15 in order), then the lanes are summed
 * 0..7 in order. */
float orc_sq_dist(const float *p, const float *r) {
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < DESC_LEN / 8; c++) {
        for (int k = 0; k < 8; k++) {
            float t = p[8 * c + k] - r[8 * c + k];
            float tt = t * t;
            acc[k] = acc[k] + tt;
        }
    }
    float s = -0.0f;
    for (int k = 0; k < 8; k++) s = s + acc[k];
    return s;
}

/* matching.rs:2373-2377: fold(0, |s, (u, v)| s + (u - v) * (u - v)). Also the
 * per-pair sum of ratio_match_reference (:1607-1612, powi(2) == x*x). */
float orc_sq_dist_seq(const float *p, const float *r) {
    float s = 0.0f;
    for (int k = 0; k < DESC_LEN; k++) {
        float t = p[k] - r[k];
        float tt = t * t;
        s = s + tt;
    }
    return s;
}

/* FP64 distance from the same f32 inputs (error reporting only). */
double orc_sq_dist_f64(const float *p, const float *r) {
    double s = 0.0;
    for (int k = 0; k < DESC_LEN; k++) {
        double t = (double)p[k] - (double)r[k];
        s += t * t;
    }
    return s;
}

void orc_dist_matrix(const float *a, int64_t na, const float *b, int64_t nb, float *out) {
    for (int64_t i = 0; i < na; i++)
        for (int64_t j = 0; j < nb; j++) out[i * nb + j] = orc_sq_dist(a + i * DESC_LEN, b + j * DESC_LEN);
}

void orc_dist_matrix_f64(const float *a, int64_t na, const float *b, int64_t nb, double *out) {
    for (int64_t i = 0; i < na; i++)
        for (int64_t j = 0; j < nb; j++) out[i * nb + j] = orc_sq_dist_f64(a + i * DESC_LEN, b + j * DESC_LEN);
}

/* --------------------------------------------------------- ratio_match */

typedef struct {
    uint64_t j1; /* usize::MAX when unset */
    float d1, d2;
} row_state;

typedef struct {
    float d;
    uint64_t i;
} col_state;

typedef struct {
    const float *a, *b;
    int64_t na, nb;
    int mutual;
    row_state *rows;   /* na */
    col_state *cols;   /* nblocks * nb (mutual only) */
    int64_t nblocks;
    int64_t next;      /* shared block counter */
    pthread_mutex_t mu;
} rm_job;

/* One 64-row block: matching.rs:171-193 (j outer, r inner; strict `<` updates). */
static void rm_block(rm_job *J, int64_t bi) {
    int64_t r0 = bi * MATCH_BLOCK;
    int64_t rn = J->na - r0 < MATCH_BLOCK ? J->na - r0 : MATCH_BLOCK;
    row_state *row = J->rows + r0;
    col_state *col = J->mutual ? J->cols + bi * J->nb : NULL;
    for (int64_t r = 0; r < rn; r++) {
        row[r].j1 = UINT64_MAX;
        row[r].d1 = INFINITY;
        row[r].d2 = INFINITY;
    }
    if (col)
        for (int64_t j = 0; j < J->nb; j++) {
            col[j].d = INFINITY;
            col[j].i = UINT64_MAX;
        }
    for (int64_t j = 0; j < J->nb; j++) {
        const float *fb = J->b + j * DESC_LEN;
        for (int64_t r = 0; r < rn; r++) {
            float d = orc_sq_dist(J->a + (r0 + r) * DESC_LEN, fb);
            row_state *best = &row[r];
            if (d < best->d1) {
                best->d2 = best->d1;
                best->d1 = d;
                best->j1 = (uint64_t)j;
            } else if (d < best->d2) {
                best->d2 = d;
            }
            if (col && d < col[j].d) {
                col[j].d = d;
                col[j].i = (uint64_t)(r0 + r);
            }
        }
    }
}

static void *rm_worker(void *arg) {
    rm_job *J = (rm_job *)arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int64_t bi = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (bi >= J->nblocks) break;
        rm_block(J, bi);
    }
    return NULL;
}

/* matching.rs:167-215. Writes (i, j) pairs in ascending i to out (capacity
 * >= na pairs, 2*na uint32) and returns their count. nthreads <= 1 runs serially. */
int64_t orc_ratio_match(const float *a, int64_t na, const float *b, int64_t nb, float ratio, int mutual,
                        int nthreads, uint32_t *out) {
    if (na <= 0) return 0;
    rm_job J;
    J.a = a;
    J.b = b;
    J.na = na;
    J.nb = nb;
    J.mutual = mutual;
    J.nblocks = (na + MATCH_BLOCK - 1) / MATCH_BLOCK;
    J.rows = (row_state *)malloc(sizeof(row_state) * (size_t)na);
    J.cols = mutual && nb > 0 ? (col_state *)malloc(sizeof(col_state) * (size_t)(J.nblocks * nb)) : NULL;
    J.next = 0;
    pthread_mutex_init(&J.mu, NULL);
    if (nthreads <= 1 || J.nblocks == 1) {
        for (int64_t bi = 0; bi < J.nblocks; bi++) rm_block(&J, bi);
    } else {
        int nt = nthreads < J.nblocks ? nthreads : (int)J.nblocks;
        pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nt);
        for (int t = 0; t < nt; t++) pthread_create(&th[t], NULL, rm_worker, &J);
        for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
        free(th);
    }
    pthread_mutex_destroy(&J.mu);
    /* :196-203: merge column bests block by block, strict `<`. */
    col_state *best = NULL;
    if (mutual && nb > 0) {
        best = (col_state *)malloc(sizeof(col_state) * (size_t)nb);
        for (int64_t j = 0; j < nb; j++) {
            best[j].d = INFINITY;
            best[j].i = UINT64_MAX;
        }
        for (int64_t bi = 0; bi < J.nblocks; bi++)
            for (int64_t j = 0; j < nb; j++)
                if (J.cols[bi * nb + j].d < best[j].d) best[j] = J.cols[bi * nb + j];
    }
    /* :204-214: ratio and mutual filter. */
    float r2 = ratio * ratio;
    int64_t n = 0;
    for (int64_t i = 0; i < na; i++) {
        row_state s = J.rows[i];
        if (s.j1 == UINT64_MAX || !isfinite(s.d2) || s.d1 >= r2 * s.d2) continue;
        if (mutual && best[s.j1].i != (uint64_t)i) continue;
        out[2 * n] = (uint32_t)i;
        out[2 * n + 1] = (uint32_t)s.j1;
        n++;
    }
    free(J.rows);
    free(J.cols);
    free(best);
    return n;
}

/* Exact per-row (j1, d1, d2) and per-column (i1, d) states of ratio_match,
 * exposed so tests can explain a mismatch. j1/i1 = UINT32_MAX when unset. */
void orc_ratio_states(const float *a, int64_t na, const float *b, int64_t nb, uint32_t *row_j1, float *row_d1,
                      float *row_d2, uint32_t *col_i1, float *col_d) {
    for (int64_t j = 0; j < nb; j++) {
        col_i1[j] = UINT32_MAX;
        col_d[j] = INFINITY;
    }
    for (int64_t i = 0; i < na; i++) {
        uint32_t j1 = UINT32_MAX;
        float d1 = INFINITY, d2 = INFINITY;
        for (int64_t j = 0; j < nb; j++) {
            float d = orc_sq_dist(a + i * DESC_LEN, b + j * DESC_LEN);
            if (d < d1) {
                d2 = d1;
                d1 = d;
                j1 = (uint32_t)j;
            } else if (d < d2) {
                d2 = d;
            }
            if (d < col_d[j]) {
                col_d[j] = d;
                col_i1[j] = (uint32_t)i;
            }
        }
        row_j1[i] = j1;
        row_d1[i] = d1;
        row_d2[i] = d2;
    }
}

/* matching.rs:1597-1636 (`ratio_match_reference`): per row a full scan of b
 * with the sequential sum; when mutual, the reverse scan of a from b[j]. */
static int nearest_seq(const float *q, const float *set, int64_t n, uint64_t *j1, float *d1, float *d2) {
    uint64_t bj = UINT64_MAX;
    float b1 = INFINITY, b2 = INFINITY;
    for (int64_t j = 0; j < n; j++) {
        float d = orc_sq_dist_seq(q, set + j * DESC_LEN);
        if (d < b1) {
            b2 = b1;
            b1 = d;
            bj = (uint64_t)j;
        } else if (d < b2) {
            b2 = d;
        }
    }
    *j1 = bj;
    *d1 = b1;
    *d2 = b2;
    return bj != UINT64_MAX;
}

int64_t orc_ratio_match_naive(const float *a, int64_t na, const float *b, int64_t nb, float ratio, int mutual,
                              uint32_t *out) {
    int64_t n = 0;
    float r2 = ratio * ratio;
    for (int64_t i = 0; i < na; i++) {
        uint64_t j1;
        float d1, d2;
        if (!nearest_seq(a + i * DESC_LEN, b, nb, &j1, &d1, &d2)) continue;
        if (!isfinite(d2) || d1 >= r2 * d2) continue;
        if (mutual) {
            uint64_t i1;
            float e1, e2;
            if (!nearest_seq(b + j1 * DESC_LEN, a, na, &i1, &e1, &e2) || i1 != (uint64_t)i) continue;
        }
        out[2 * n] = (uint32_t)i;
        out[2 * n + 1] = (uint32_t)j1;
        n++;
    }
    return n;
}

/* matching.rs:1866-1878: FNV-1a 64 over (i as u64, j as u64) little-endian bytes. */
uint64_t orc_pairs_hash(const uint32_t *pairs, int64_t n) {
    uint64_t h = 0xcbf29ce484222325ULL;
    for (int64_t p = 0; p < 2 * n; p++) {
        uint64_t v = pairs[p];
        for (int b = 0; b < 8; b++) {
            h ^= (v >> (8 * b)) & 0xff;
            h *= 0x100000001b3ULL;
        }
    }
    return h;
}

/* ------------------------------------------------------ pair generators */

static uint64_t absdiff(uint64_t x, uint64_t y) { return x > y ? x - y : y - x; }
static int is_pow2(uint64_t d) { return d != 0 && (d & (d - 1)) == 0; }

/* matching.rs:14-40. views: 2*nv (cam, pos). Writes up to cap pairs and
 * returns the total count (which may exceed cap). */
int64_t orc_candidate_pairs(const uint64_t *views, int64_t nv, uint64_t temporal, uint64_t cross, uint64_t pow2_max,
                            uint32_t *out, int64_t cap) {
    int64_t n = 0;
    for (int64_t i = 0; i < nv; i++)
        for (int64_t j = i + 1; j < nv; j++) {
            uint64_t ca = views[2 * i], pa = views[2 * i + 1], cb = views[2 * j], pb = views[2 * j + 1];
            uint64_t d = absdiff(pa, pb);
            int ok = ca == cb ? (d >= 1 && (d <= temporal || (is_pow2(d) && d <= pow2_max))) : (d <= cross);
            if (ok) {
                if (n < cap) {
                    out[2 * n] = (uint32_t)i;
                    out[2 * n + 1] = (uint32_t)j;
                }
                n++;
            }
        }
    return n;
}

static int pair_cmp(const void *x, const void *y) {
    const uint32_t *p = (const uint32_t *)x, *q = (const uint32_t *)y;
    if (p[0] != q[0]) return p[0] < q[0] ? -1 : 1;
    if (p[1] != q[1]) return p[1] < q[1] ? -1 : 1;
    return 0;
}

/* matching.rs:103-142. spec != 0: CrossSchedule::Spec{range = spec_range};
 * else CrossSchedule::Formation{right_min, left_min, max, step}. Cameras:
 * front 0, right 1, left 2 (:42-45). Returns the count (sorted, unique). */
int64_t orc_scheduled_pairs(const uint64_t *views, int64_t nv, uint64_t temporal, uint64_t pow2_max, int spec,
                            uint64_t spec_range, uint64_t right_min, uint64_t left_min, uint64_t max,
                            uint64_t step, uint32_t *out, int64_t cap) {
    int64_t n = 0, alloc = 1024;
    uint32_t *buf = (uint32_t *)malloc(sizeof(uint32_t) * 2 * (size_t)alloc);
    for (int64_t i = 0; i < nv; i++)
        for (int64_t j = 0; j < nv; j++) {
            if (i == j) continue;
            uint64_t ca = views[2 * i], pa = views[2 * i + 1], cb = views[2 * j], pb = views[2 * j + 1];
            uint64_t d = absdiff(pa, pb);
            int ok;
            if (ca == cb) {
                ok = j > i && d >= 1 && (d <= temporal || (is_pow2(d) && d <= pow2_max));
            } else if (spec) {
                ok = j > i && d <= spec_range;
            } else {
                int has = 0;
                uint64_t lo = 0;
                if (ca == 0 && cb == 1) { has = 1; lo = right_min; }
                if (ca == 0 && cb == 2) { has = 1; lo = left_min; }
                uint64_t st = step > 1 ? step : 1;
                ok = has && pb >= pa + lo && pb <= pa + max && (pb - pa - lo) % st == 0;
            }
            if (ok) {
                if (n == alloc) {
                    alloc *= 2;
                    buf = (uint32_t *)realloc(buf, sizeof(uint32_t) * 2 * (size_t)alloc);
                }
                buf[2 * n] = (uint32_t)(i < j ? i : j);
                buf[2 * n + 1] = (uint32_t)(i < j ? j : i);
                n++;
            }
        }
    qsort(buf, (size_t)n, 2 * sizeof(uint32_t), pair_cmp);
    int64_t u = 0;
    for (int64_t k = 0; k < n; k++) {
        if (u > 0 && buf[2 * k] == buf[2 * (u - 1)] && buf[2 * k + 1] == buf[2 * (u - 1) + 1]) continue;
        buf[2 * u] = buf[2 * k];
        buf[2 * u + 1] = buf[2 * k + 1];
        u++;
    }
    for (int64_t k = 0; k < u && k < cap; k++) {
        out[2 * k] = buf[2 * k];
        out[2 * k + 1] = buf[2 * k + 1];
    }
    free(buf);
    return u;
}

/* Serial loop over image pairs, each matched with orc_ratio_match using
 * nthreads (benches/pipeline.rs:247-253). desc holds all views back to back;
 * view_off[v] is the first row of view v, view_n[v] its row count. Returns the
 * total number of matches; counts[p] receives each pair's count. */
int64_t orc_match_pairs(const float *desc, const int64_t *view_off, const int64_t *view_n, const uint32_t *pairs,
                        int64_t npairs, float ratio, int mutual, int nthreads, int64_t *counts) {
    int64_t total = 0, cap = 0;
    uint32_t *tmp = NULL;
    for (int64_t p = 0; p < npairs; p++) {
        uint32_t u = pairs[2 * p], v = pairs[2 * p + 1];
        if (view_n[u] > cap) {
            cap = view_n[u];
            tmp = (uint32_t *)realloc(tmp, sizeof(uint32_t) * 2 * (size_t)cap);
        }
        int64_t c = orc_ratio_match(desc + view_off[u] * DESC_LEN, view_n[u], desc + view_off[v] * DESC_LEN,
                                    view_n[v], ratio, mutual, nthreads, tmp);
        if (counts) counts[p] = c;
        total += c;
    }
    free(tmp);
    return total;
}

/* ------------------------------------------------------ Sampson scoring */

/* two_view.rs:456-465, in f64 and in the operation order of the reference's
 * linear algebra (nalgebra 0.33.3, Cargo.lock), as its published source
 * states it (the crate's source is not part of the reference, so this order
 * is a restatement, not checked against the reference's own outputs):
 *   - Matrix3 * Vector3 is a gemv that adds the columns in order: row i of
 *     y = e p is ((e[i][0] * p0 + e[i][1] * p1) + e[i][2] * p2), every product
 *     and sum rounded separately (Rust does not contract to FMA);
 *   - e.transpose() * q the same with the columns of e^T (the rows of e);
 *   - den = sqrt(((ep0^2 + ep1^2) + etq0^2) + etq1^2), left to right;
 *   - q.dot(ep) = (q0 ep0 + q1 ep1) + q2 ep2;
 *   - the residual is q.dot(ep) / den, or 0 when den is not > 0.
 * e is row-major (e[3 r + c] = E[r][c], nalgebra's Matrix3::new order);
 * p = (ax, ay, 1), q = (bx, by, 1). */
double orc_sampson_residual(const double *e, double ax, double ay, double bx, double by) {
    double ep[3], etq[3];
    for (int i = 0; i < 3; ++i) {
        double y = e[3 * i + 0] * ax;
        y = e[3 * i + 1] * ay + y;
        y = e[3 * i + 2] * 1.0 + y;
        ep[i] = y;
    }
    for (int i = 0; i < 3; ++i) {
        double y = e[0 * 3 + i] * bx;
        y = e[1 * 3 + i] * by + y;
        y = e[2 * 3 + i] * 1.0 + y;
        etq[i] = y;
    }
    const double den = sqrt(((ep[0] * ep[0] + ep[1] * ep[1]) + etq[0] * etq[0]) + etq[1] * etq[1]);
    if (den > 0.0) {
        const double dot = (bx * ep[0] + by * ep[1]) + 1.0 * ep[2];
        return dot / den;
    }
    return 0.0;
}

typedef struct {
    const double *pts, *thresh, *E;
    const uint64_t *pair_off, *mask_off;
    const uint32_t *hyp_pair;
    uint32_t *counts, *masks;
    int64_t nh, next;
    pthread_mutex_t mu;
} ss_job;

static void ss_one(ss_job *J, int64_t h) {
    const uint32_t p = J->hyp_pair[h];
    const uint64_t m0 = J->pair_off[p], m1 = J->pair_off[p + 1];
    const double th = J->thresh[p];
    const double *e = J->E + 9 * h;
    uint32_t c = 0;
    uint32_t *mk = (J->masks && J->mask_off && J->mask_off[h] != UINT64_MAX) ? J->masks + J->mask_off[h] : NULL;
    for (uint64_t i = m0; i < m1; ++i) {
        const double *q = J->pts + 4 * i;
        /* inliers_of / count_at_least: |r| < th, strict (two_view.rs:806, :812) */
        const int in = fabs(orc_sampson_residual(e, q[0], q[1], q[2], q[3])) < th;
        c += (uint32_t)in;
        if (mk) {
            const uint64_t k = i - m0;
            if ((k & 31) == 0) mk[k >> 5] = 0;
            if (in) mk[k >> 5] |= 1u << (k & 31);
        }
    }
    J->counts[h] = c;
}

static void *ss_worker(void *arg) {
    ss_job *J = (ss_job *)arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const int64_t h0 = J->next;
        J->next += 64;
        pthread_mutex_unlock(&J->mu);
        if (h0 >= J->nh) break;
        const int64_t h1 = h0 + 64 < J->nh ? h0 + 64 : J->nh;
        for (int64_t h = h0; h < h1; ++h) ss_one(J, h);
    }
    return NULL;
}

/* Every hypothesis h (E + 9 h, of pair hyp_pair[h]) scored over its pair's
 * matches pts[pair_off[p] .. pair_off[p+1]) (4 doubles each: a.x, a.y, b.x,
 * b.y): counts[h] = #{i : |r_h(i)| < thresh[p]} (the count count_at_least
 * returns when it reaches `need`, the length of inliers_of's true set), and,
 * where mask_off[h] != UINT64_MAX, the inlier bits of inliers_of at
 * masks[mask_off[h] ..] (bit i % 32 of word i / 32). Hypotheses are spread
 * over `threads` threads. */
void orc_sampson_score(const double *pts, const uint64_t *pair_off, const double *thresh, const double *E,
                       const uint32_t *hyp_pair, int64_t nh, uint32_t *counts, const uint64_t *mask_off,
                       uint32_t *masks, int threads) {
    ss_job J;
    J.pts = pts;
    J.thresh = thresh;
    J.E = E;
    J.pair_off = pair_off;
    J.mask_off = mask_off;
    J.hyp_pair = hyp_pair;
    J.counts = counts;
    J.masks = masks;
    J.nh = nh;
    J.next = 0;
    pthread_mutex_init(&J.mu, NULL);
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    int started = 0;
    for (int t = 1; t < threads; ++t)
        if (pthread_create(&th[started], NULL, ss_worker, &J) == 0) ++started;
    ss_worker(&J);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&J.mu);
}
