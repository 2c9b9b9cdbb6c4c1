/*
 * bmnd_oracle.c -- CPU restatement of the BMND direct-Poisson collaborative
 * filtering path.  TEST INFRASTRUCTURE ONLY: the checker for the GPU library
 * (tests, __graft_entry__.smoke) and the timed CPU baseline of bench.py.  The
 * product never links, loads or calls this file.
 *
 * It follows the reference cduhme/bmnd (pure Python + Numba) step by step
 * with NumPy float32 semantics: every float32 operation is rounded on its own
 * (built with -ffp-contract=off), matrix products accumulate with one fused
 * multiply-add per term in k order (what NumPy's OpenBLAS sgemm does; checked
 * bit-exact on the golden inputs), and the few float64 steps of the reference
 * stay float64.  Where the reference's own result depends on its platform
 * (NumPy's float32 log, the unstable argsort inside the exact variance) the
 * oracle uses the C library's logf and ascending entry order.
 *
 * Pinned against the reference: the tests/golden fixtures hold outputs of the
 * reference itself (run here through oracle/shim), and tests/test_oracle_*.py
 * compare this file with them.
 *
 * Build: see oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off -shared).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/bmnd_gb300.h"

#define MAXD BMND_MAX_DIMS

/* ------------------------------------------------------------------ */
/* schedule: shifts.py:229-266 (_generate_axis_shifts,                */
/* get_generated_reference_shifts) and :519-576                       */
/* ------------------------------------------------------------------ */

static int round_half_even(double x) {
    double r = nearbyint(x); /* default rounding mode: ties to even, like Python round() */
    return (int)r;
}

static int axis_shifts(int block, int step, int allow_multiple, double density, int* out) {
    if (!allow_multiple || block < 3 || step < 1 || step > block) {
        out[0] = 0;
        return 1;
    }
    double safe = density > 0.0 ? density : 0.0;
    int count = (int)ceil(safe * (double)(block - 1) / (double)step);
    if (count < 1) count = 1;
    if (count > block) count = block;
    if (count == 1) {
        out[0] = 0;
        return 1;
    }
    /* np.linspace(0, block-1, count) then sorted(set(round(x)) | {0}) */
    int present[64] = {0};
    present[0] = 1;
    double stop = (double)(block - 1);
    double delta = stop / (double)(count - 1);
    for (int i = 0; i < count; ++i) {
        double v = (i == count - 1) ? stop : (double)i * delta;
        int r = round_half_even(v);
        if (r >= 0 && r < 64) present[r] = 1;
    }
    int n = 0;
    for (int i = 0; i < 64; ++i)
        if (present[i]) out[n++] = i;
    return n;
}

int oracle_schedule(int32_t ndim, const int32_t* counts, const int32_t* block,
                    const int32_t* step, double shift_density, int32_t schedule_density,
                    int32_t* out_abs, int32_t* out_shifted, int32_t* out_shift,
                    int64_t capacity, int64_t* out_count) {
    if (ndim < 1 || ndim > MAXD) return BMND_ERR_INVALID_ARG;
    int shifts[MAXD][64];
    int nshift[MAXD];
    int last_valid[MAXD], slots[MAXD];
    int64_t total_slots = 1, grid = 1;
    for (int d = 0; d < ndim; ++d) {
        nshift[d] = axis_shifts(block[d], step[d], d < (ndim - 1 > 0 ? ndim - 1 : 0),
                                shift_density, shifts[d]);
        last_valid[d] = counts[d] - 1 > 0 ? counts[d] - 1 : 0;
        slots[d] = (last_valid[d] + step[d] - 1) / step[d] + 1;
        total_slots *= slots[d];
        grid *= (counts[d] > 0 ? counts[d] : 1);
    }
    int phases = schedule_density > 1 ? schedule_density : 1;
    uint8_t* seen = (uint8_t*)calloc((size_t)grid, 1);
    if (!seen) return BMND_ERR_WORKSPACE;
    int64_t n = 0;
    int slot[MAXD];
    for (int64_t s = 0; s < total_slots; ++s) {
        int64_t rem = s;
        for (int d = ndim - 1; d >= 0; --d) {
            slot[d] = (int)(rem % slots[d]);
            rem /= slots[d];
        }
        for (int ph = 0; ph < phases; ++ph) {
            int abs_pos[MAXD], base[MAXD], shift[MAXD];
            for (int d = 0; d < ndim; ++d) {
                int b = slot[d] * step[d];
                if (b > last_valid[d]) b = last_valid[d];
                int offset = 0;
                if (d < ndim - 1) offset = shifts[d][(slot[d + 1] + ph) % nshift[d]];
                int a = b - offset;
                if (a < 0) a = 0;
                if (a > last_valid[d]) a = last_valid[d];
                if (slot[d] == slots[d] - 1) a = last_valid[d];
                base[d] = b;
                abs_pos[d] = a;
                shift[d] = b - a;
            }
            int64_t lin = 0;
            for (int d = 0; d < ndim; ++d) lin = lin * (counts[d] > 0 ? counts[d] : 1) + abs_pos[d];
            if (seen[lin]) continue;
            seen[lin] = 1;
            if (n < capacity) {
                for (int d = 0; d < ndim; ++d) {
                    if (out_abs) out_abs[n * ndim + d] = abs_pos[d];
                    if (out_shifted) out_shifted[n * ndim + d] = base[d];
                    if (out_shift) out_shift[n * ndim + d] = shift[d];
                }
            }
            ++n;
        }
    }
    free(seen);
    *out_count = n;
    return BMND_OK;
}

/* ------------------------------------------------------------------ */
/* distances: blockmatching.py:322-371                                */
/* ------------------------------------------------------------------ */

float oracle_patch_distance(const float* ref, const float* cand, int P, int code,
                            double count_scale) {
    float d = 0.0f;
    if (code == BMND_DIST_SSD) {
        for (int p = 0; p < P; ++p) {
            float diff = cand[p] - ref[p];
            d = d + diff * diff;
        }
        return d;
    }
    float inv = (float)(1.0 / count_scale);
    for (int p = 0; p < P; ++p) {
        float r = ref[p] * inv;
        if (r < 0.0f) r = 0.0f;
        float c = cand[p] * inv;
        if (c < 0.0f) c = 0.0f;
        if (code == BMND_DIST_POISSON_DEVIANCE) {
            float s = r + c;
            if (s > 0.0f) {
                float contrib = 0.0f;
                if (r > 0.0f) contrib = contrib + r * logf(2.0f * r / s);
                if (c > 0.0f) contrib = contrib + c * logf(2.0f * c / s);
                d = d + 2.0f * contrib;
            }
        } else if (code == BMND_DIST_PEARSON) {
            float s = r + c;
            if (s > 0.0f) {
                float diff = c - r;
                d = d + diff * diff / s;
            }
        } else {
            float rs = 2.0f * sqrtf(r + 0.375f);
            float cs = 2.0f * sqrtf(c + 0.375f);
            float diff = cs - rs;
            d = d + 0.5f * diff * diff;
        }
    }
    if (d < 0.0f) d = 0.0f;
    return d / (float)P;
}

/* float64 restatement (what Numba's type unification computes) */
double oracle_patch_distance_f64(const float* ref, const float* cand, int P, int code,
                                 double count_scale) {
    double d = 0.0;
    if (code == BMND_DIST_SSD) {
        for (int p = 0; p < P; ++p) {
            double diff = (double)cand[p] - (double)ref[p];
            d += diff * diff;
        }
        return d;
    }
    double inv = 1.0 / count_scale;
    for (int p = 0; p < P; ++p) {
        double r = ref[p] * inv;
        if (r < 0.0) r = 0.0;
        double c = cand[p] * inv;
        if (c < 0.0) c = 0.0;
        if (code == BMND_DIST_POISSON_DEVIANCE) {
            double s = r + c;
            if (s > 0.0) {
                double contrib = 0.0;
                if (r > 0.0) contrib += r * log(2.0 * r / s);
                if (c > 0.0) contrib += c * log(2.0 * c / s);
                d += 2.0 * contrib;
            }
        } else if (code == BMND_DIST_PEARSON) {
            double s = r + c;
            if (s > 0.0) d += (c - r) * (c - r) / s;
        } else {
            double diff = 2.0 * sqrt(c + 0.375) - 2.0 * sqrt(r + 0.375);
            d += 0.5 * diff * diff;
        }
    }
    if (d < 0.0) d = 0.0;
    return d / (double)P;
}

/* blockmatching.py:957-964 */
float oracle_canonical(float d) {
    if (!isfinite(d)) return d;
    double mag = fabs((double)d);
    if (mag < 1.0) mag = 1.0;
    double e = floor(log2(mag));
    double quantum = 32.0 * (double)1.1920928955078125e-07 * pow(2.0, e);
    return (float)(nearbyint((double)d / quantum) * quantum);
}

/* ------------------------------------------------------------------ */
/* block matching: blockmatching.py:913-954, :967-1205                */
/* ------------------------------------------------------------------ */

typedef struct {
    int ndim;
    int counts[MAXD];
    int radius[MAXD];
    int max_m, min_m, pow2, code, stab;
    double scale;
    /* patch source: either a table or a volume view */
    const float* table;
    int patch_vol;
    const float* volume;
    int shape[MAXD];
    int block[MAXD];
    int use_f64;
    /* Poisson SSD noise bias (blockmatching.py:1140-1145, :432-443): gamma
     * and the count scale, both float32 as they meet the float32 patches */
    int poisson_bias;
    float bias_gamma, bias_scale;
} match_ctx;

static void get_patch(const match_ctx* m, int64_t lin, float* out) {
    if (m->table) {
        memcpy(out, m->table + lin * m->patch_vol, sizeof(float) * (size_t)m->patch_vol);
        return;
    }
    int q[MAXD];
    int64_t rem = lin;
    for (int d = m->ndim - 1; d >= 0; --d) {
        q[d] = (int)(rem % m->counts[d]);
        rem /= m->counts[d];
    }
    int idx = 0;
    if (m->ndim == 1) {
        for (int a = 0; a < m->block[0]; ++a) out[idx++] = m->volume[q[0] + a];
    } else if (m->ndim == 2) {
        for (int a = 0; a < m->block[0]; ++a)
            for (int b = 0; b < m->block[1]; ++b)
                out[idx++] = m->volume[(int64_t)(q[0] + a) * m->shape[1] + q[1] + b];
    } else {
        for (int a = 0; a < m->block[0]; ++a)
            for (int b = 0; b < m->block[1]; ++b)
                for (int c = 0; c < m->block[2]; ++c)
                    out[idx++] = m->volume[((int64_t)(q[0] + a) * m->shape[1] + q[1] + b) *
                                               m->shape[2] +
                                           q[2] + c];
    }
}

typedef struct {
    float key;
    int64_t lin;
} cand_t;

static int precedes(float k1, int64_t l1, float k2, int64_t l2) {
    if (k1 < k2) return 1;
    if (k1 > k2) return 0;
    return l1 < l2;
}

static int insert_limited(cand_t* buf, int size, int limit, float key, int64_t lin) {
    if (limit == 0) return size;
    int at;
    if (size < limit) {
        ++size;
        at = size - 1;
    } else {
        if (!precedes(key, lin, buf[limit - 1].key, buf[limit - 1].lin)) return size;
        at = limit - 1;
    }
    while (at > 0 && precedes(key, lin, buf[at - 1].key, buf[at - 1].lin)) {
        buf[at] = buf[at - 1];
        --at;
    }
    buf[at].key = key;
    buf[at].lin = lin;
    return size;
}

static int largest_pow2_at_most(int v) {
    if (v <= 0) return 0;
    int p = 1;
    while ((p << 1) <= v) p <<= 1;
    return p;
}

static void match_one(const match_ctx* m, const int32_t* center, float threshold, int32_t* sel,
                      int32_t* count, int32_t* accepted_out, float* refp, float* candp) {
    int ndim = m->ndim;
    int64_t center_lin = 0;
    int lo[MAXD], ext[MAXD], coord[MAXD];
    for (int d = 0; d < ndim; ++d) center_lin = center_lin * m->counts[d] + center[d];
    for (int d = 0; d < ndim; ++d) {
        int l = center[d] - m->radius[d];
        if (l < 0) l = 0;
        int h = center[d] + m->radius[d];
        if (h > m->counts[d] - 1) h = m->counts[d] - 1;
        lo[d] = l;
        ext[d] = h - l + 1;
        coord[d] = l;
    }
    int P = m->table ? m->patch_vol : 1;
    if (!m->table) {
        P = 1;
        for (int d = 0; d < ndim; ++d) P *= m->block[d];
    }
    get_patch(m, center_lin, refp);
    int required = m->min_m < m->max_m ? m->min_m : m->max_m;
    cand_t acc[BMND_MAX_STACK + 1], rej[BMND_MAX_STACK + 1];
    int acc_n = 0, rej_n = 0, accepted = 0;
    int stab = m->stab && m->code != BMND_DIST_SSD;
    float tkey = stab ? oracle_canonical(threshold) : threshold;
    int done = 0;
    while (!done) {
        int64_t lin = coord[0];
        for (int d = 1; d < ndim; ++d) lin = lin * m->counts[d] + coord[d];
        get_patch(m, lin, candp);
        float dist;
        if (m->use_f64)
            dist = (float)oracle_patch_distance_f64(refp, candp, P, m->code, m->scale);
        else
            dist = oracle_patch_distance(refp, candp, P, m->code, m->scale);
        if (m->poisson_bias && lin != center_lin) {
            /* sum over r + c > 0 of scale * (r + c), float32 in patch order */
            float bias = 0.0f;
            for (int p = 0; p < P; ++p) {
                float pooled = refp[p] + candp[p];
                if (pooled > 0.0f) bias = bias + m->bias_scale * pooled;
            }
            dist = dist - m->bias_gamma * bias;
        }
        float key = stab ? oracle_canonical(dist) : dist;
        if (key < tkey) {
            ++accepted;
            acc_n = insert_limited(acc, acc_n, m->max_m, key, lin);
        } else {
            rej_n = insert_limited(rej, rej_n, required, key, lin);
        }
        for (int d = ndim - 1; d >= 0; --d) {
            coord[d] += 1;
            if (coord[d] < lo[d] + ext[d]) break;
            coord[d] = lo[d];
            if (d == 0) done = 1;
        }
    }
    int64_t selected[2 * BMND_MAX_STACK + 2];
    int sel_n = acc_n;
    for (int i = 0; i < acc_n; ++i) selected[i] = acc[i].lin;
    if (sel_n < required) {
        int need = required - sel_n;
        int take = need < rej_n ? need : rej_n;
        for (int i = 0; i < take; ++i) selected[sel_n++] = rej[i].lin;
    }
    /* _finalize_selected_lin_indices_numba */
    int64_t out[BMND_MAX_STACK];
    int n = 0;
    if (m->max_m > 0) {
        out[0] = center_lin;
        n = 1;
        for (int i = 0; i < sel_n && n < m->max_m; ++i) {
            int64_t l = selected[i];
            if (l < 0 || l == center_lin) continue;
            int seen = 0;
            for (int j = 0; j < n; ++j)
                if (out[j] == l) seen = 1;
            if (!seen) out[n++] = l;
        }
        if (m->pow2 && n > 0) {
            int target = largest_pow2_at_most(n);
            if (m->min_m > target) target = m->min_m;
            if (target < n) n = target;
        }
    }
    for (int i = 0; i < m->max_m; ++i) sel[i] = i < n ? (int32_t)out[i] : -1;
    *count = n;
    *accepted_out = accepted;
}

static int run_match(const match_ctx* m, const int32_t* refs, int64_t n_refs,
                     const float* thresholds, int32_t* sel, int32_t* count, int32_t* accepted,
                     int threads) {
    int P = m->table ? m->patch_vol : 1;
    if (!m->table)
        for (int d = 0; d < m->ndim; ++d) P *= m->block[d];
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
#endif
    {
        float* refp = (float*)malloc(sizeof(float) * (size_t)P);
        float* candp = (float*)malloc(sizeof(float) * (size_t)P);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t i = 0; i < n_refs; ++i)
            match_one(m, refs + i * m->ndim, thresholds[i], sel + i * m->max_m, count + i,
                      accepted + i, refp, candp);
        free(refp);
        free(candp);
    }
    (void)threads;
    return BMND_OK;
}

int oracle_blockmatch_patches(const BmndMatchParams* p, const float* patches, int32_t patch_vol,
                              const int32_t* refs, int64_t n_refs, const float* thresholds,
                              int32_t* sel, int32_t* count, int32_t* accepted, int32_t use_f64,
                              int32_t threads) {
    match_ctx m;
    memset(&m, 0, sizeof(m));
    m.ndim = p->ndim;
    for (int d = 0; d < p->ndim; ++d) {
        m.counts[d] = p->counts[d];
        m.radius[d] = p->search_radius[d];
    }
    m.max_m = p->max_matches;
    m.min_m = p->min_matches;
    m.pow2 = p->prefer_power_of_two;
    m.code = p->distance;
    m.stab = p->stabilize_ties;
    m.scale = p->distance == BMND_DIST_SSD ? 1.0 : p->count_scale;
    m.table = patches;
    m.patch_vol = patch_vol;
    m.use_f64 = use_f64;
    return run_match(&m, refs, n_refs, thresholds, sel, count, accepted, threads);
}

/* oracle_blockmatch_volume with the Poisson SSD noise bias when gamma != 0
 * (p->distance SSD, p->count_scale the profile's poisson_count_scale) */
int oracle_blockmatch_volume_biased(const BmndMatchParams* p, const float* volume, const int32_t* shape,
                                    const int32_t* block, const int32_t* refs, int64_t n_refs,
                                    const float* thresholds, float gamma, int32_t* sel, int32_t* count,
                                    int32_t* accepted, int32_t threads) {
    match_ctx m;
    memset(&m, 0, sizeof(m));
    m.ndim = p->ndim;
    for (int d = 0; d < p->ndim; ++d) {
        m.counts[d] = p->counts[d];
        m.radius[d] = p->search_radius[d];
        m.shape[d] = shape[d];
        m.block[d] = block[d];
    }
    m.max_m = p->max_matches;
    m.min_m = p->min_matches;
    m.pow2 = p->prefer_power_of_two;
    m.code = p->distance;
    m.stab = p->stabilize_ties;
    m.scale = 1.0;
    m.volume = volume;
    m.poisson_bias = p->distance == BMND_DIST_SSD && gamma != 0.0f;
    m.bias_gamma = gamma;
    m.bias_scale = (float)p->count_scale;
    return run_match(&m, refs, n_refs, thresholds, sel, count, accepted, threads);
}

int oracle_blockmatch_volume(const BmndMatchParams* p, const float* volume, const int32_t* shape,
                             const int32_t* block, const int32_t* refs, int64_t n_refs,
                             const float* thresholds, int32_t* sel, int32_t* count,
                             int32_t* accepted, int32_t use_f64, int32_t threads) {
    match_ctx m;
    memset(&m, 0, sizeof(m));
    m.ndim = p->ndim;
    for (int d = 0; d < p->ndim; ++d) {
        m.counts[d] = p->counts[d];
        m.radius[d] = p->search_radius[d];
        m.shape[d] = shape[d];
        m.block[d] = block[d];
    }
    m.max_m = p->max_matches;
    m.min_m = p->min_matches;
    m.pow2 = p->prefer_power_of_two;
    m.code = p->distance;
    m.stab = p->stabilize_ties;
    m.scale = p->distance == BMND_DIST_SSD ? 1.0 : p->count_scale;
    m.volume = volume;
    m.use_f64 = use_f64;
    return run_match(&m, refs, n_refs, thresholds, sel, count, accepted, threads);
}

/* ------------------------------------------------------------------ */
/* transforms: transforms.py:359-440 and the matrix product rule      */
/* ------------------------------------------------------------------ */

/* hierarchical Haar (transforms.py:393-408), built the same way in float32 */
static void haar_matrix(int n, float* out) {
    float* cur = (float*)malloc(sizeof(float) * (size_t)n * (size_t)n);
    float* nxt = (float*)malloc(sizeof(float) * (size_t)n * (size_t)n);
    const float s = (float)(1.0 / sqrt(2.0));
    cur[0] = 1.0f;
    int size = 1;
    while (size < n) {
        int ns = 2 * size;
        /* coarse = kron(cur, [s, s]) : size x ns */
        for (int i = 0; i < size; ++i)
            for (int j = 0; j < size; ++j) {
                nxt[i * ns + 2 * j] = cur[i * size + j] * s;
                nxt[i * ns + 2 * j + 1] = cur[i * size + j] * s;
            }
        /* detail = kron(eye(size), [s, -s]) */
        for (int i = 0; i < size; ++i)
            for (int j = 0; j < ns; ++j) nxt[(size + i) * ns + j] = 0.0f;
        for (int i = 0; i < size; ++i) {
            nxt[(size + i) * ns + 2 * i] = 1.0f * s;
            nxt[(size + i) * ns + 2 * i + 1] = 1.0f * -s;
        }
        float* t = cur;
        cur = nxt;
        nxt = t;
        size = ns;
    }
    memcpy(out, cur, sizeof(float) * (size_t)n * (size_t)n);
    free(cur);
    free(nxt);
}

/* orthonormal DCT-II, float64 formula stored as float32 (transforms.py:362-372) */
static void dct_matrix(int n, float* out) {
    const double pi = 3.14159265358979323846;
    for (int f = 0; f < n; ++f)
        for (int s = 0; s < n; ++s) {
            double norm = f == 0 ? sqrt(1.0 / n) : sqrt(2.0 / n);
            out[f * n + s] = (float)(norm * cos(pi * (s + 0.5) * f / n));
        }
}

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static void group_matrix(int kind, int n, float* fwd, float* inv) {
    if (kind == BMND_GROUP_NONE) {
        for (int i = 0; i < n * n; ++i) fwd[i] = 0.0f;
        for (int i = 0; i < n; ++i) fwd[i * n + i] = 1.0f;
    } else if (kind == BMND_GROUP_HAAR && is_pow2(n)) {
        haar_matrix(n, fwd);
    } else {
        dct_matrix(n, fwd);
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) inv[i * n + j] = fwd[j * n + i];
}

/* ------------------------------------------------------------------ */
/* filtering arithmetic type                                          */
/* ------------------------------------------------------------------ */
/* The default build rounds every filtering operation to float32, as the
   reference does.  Built with -DORACLE_F64 (libbmnd_oracle_f64.so) the same
   code carries transforms, noise statistics, shrinkage, weights, aggregation
   and the final division in float64 on the same float32 transform matrices:
   the reference's algorithm without its float32 rounding, against which the
   per-stage error of a float32 implementation is measured.  Matching is
   float32 in both builds (its decisions define the groups). */
#ifdef ORACLE_F64
typedef double real;
#define RFMA fma
#define RSQRT sqrt
#define RABS fabs
#else
typedef float real;
#define RFMA fmaf
#define RSQRT sqrtf
#define RABS fabsf
#endif

/* out = M (applied along one axis) in, with one fused multiply-add per term
   in k order.  data: dims[0..nd-1] C order; axis a has extent dims[a] == m. */
static void apply_axis(const real* in, real* out, const int* dims, int nd, int axis,
                       const real* M) {
    int m = dims[axis];
    int64_t outer = 1, inner = 1;
    for (int d = 0; d < axis; ++d) outer *= dims[d];
    for (int d = axis + 1; d < nd; ++d) inner *= dims[d];
    for (int64_t o = 0; o < outer; ++o)
        for (int i = 0; i < m; ++i)
            for (int64_t t = 0; t < inner; ++t) {
                real acc = 0;
                for (int k = 0; k < m; ++k)
                    acc = RFMA(M[i * m + k], in[(o * m + k) * inner + t], acc);
                out[(o * m + i) * inner + t] = acc;
            }
}

/* ------------------------------------------------------------------ */
/* group filtering                                                    */
/* ------------------------------------------------------------------ */

typedef struct {
    const BmndStageParams* sp;
    int P;
    int counts[MAXD];
    real gfwd[BMND_MAX_STACK + 1][BMND_MAX_STACK * BMND_MAX_STACK];
    real ginv[BMND_MAX_STACK + 1][BMND_MAX_STACK * BMND_MAX_STACK];
    real sfwd[MAXD][BMND_MAX_EDGE * BMND_MAX_EDGE];
    real sinv[MAXD][BMND_MAX_EDGE * BMND_MAX_EDGE];
    real* S; /* kron of spatial forward matrices, P x P */
} stage_ctx;

static void gather_patch(const real* vol, const int* shape, const int* block, int ndim,
                         const int* pos, real* out) {
    int idx = 0;
    if (ndim == 1) {
        for (int a = 0; a < block[0]; ++a) out[idx++] = vol[pos[0] + a];
    } else if (ndim == 2) {
        for (int a = 0; a < block[0]; ++a)
            for (int b = 0; b < block[1]; ++b)
                out[idx++] = vol[(int64_t)(pos[0] + a) * shape[1] + pos[1] + b];
    } else {
        for (int a = 0; a < block[0]; ++a)
            for (int b = 0; b < block[1]; ++b)
                for (int c = 0; c < block[2]; ++c)
                    out[idx++] =
                        vol[((int64_t)(pos[0] + a) * shape[1] + pos[1] + b) * shape[2] + pos[2] + c];
    }
}

static real variance_value(float x, const BmndStageParams* sp) {
    /* variance.py:581-585: max(scale * max(x, 0), floor) */
    real nn = x > 0.0f ? (real)x : (real)0;
    real v = (real)sp->count_scale * nn;
    real fl = (real)sp->variance_floor;
    return v > fl ? v : fl;
}

/* forward / inverse separable transform of an (n, block...) group */
static void transform_group(const stage_ctx* c, int n, const real* in, real* out, real* tmp,
                            int inverse) {
    const BmndStageParams* sp = c->sp;
    int dims[MAXD + 1];
    dims[0] = n;
    for (int d = 0; d < sp->ndim; ++d) dims[1 + d] = sp->block[d];
    int total = n * c->P;
    memcpy(tmp, in, sizeof(real) * (size_t)total);
    real* a = tmp;
    real* b = out;
    const real* G = inverse ? c->ginv[n] : c->gfwd[n];
    if (sp->group_transform != BMND_GROUP_NONE) {
        apply_axis(a, b, dims, sp->ndim + 1, 0, G);
        real* t = a;
        a = b;
        b = t;
    }
    for (int d = 0; d < sp->ndim; ++d) {
        const real* M = inverse ? c->sinv[d] : c->sfwd[d];
        apply_axis(a, b, dims, sp->ndim + 1, d + 1, M);
        real* t = a;
        a = b;
        b = t;
    }
    if (a != out) memcpy(out, a, sizeof(real) * (size_t)total);
}

/* approximate variance: squared transforms applied to the variance group
   (variance.py:613-623, :1647-1653); returns variance (not yet sqrt) */
static void approx_variance(const stage_ctx* c, int n, const real* vg, real* out, real* tmp) {
    const BmndStageParams* sp = c->sp;
    int dims[MAXD + 1];
    dims[0] = n;
    for (int d = 0; d < sp->ndim; ++d) dims[1 + d] = sp->block[d];
    int total = n * c->P;
    real* a = tmp;
    real* b = out;
    for (int i = 0; i < total; ++i) a[i] = vg[i] > 0 ? vg[i] : (real)0;
    real sq[BMND_MAX_STACK * BMND_MAX_STACK] = {0};
    if (sp->group_transform != BMND_GROUP_NONE) {
        for (int i = 0; i < n * n; ++i) sq[i] = c->gfwd[n][i] * c->gfwd[n][i];
        apply_axis(a, b, dims, sp->ndim + 1, 0, sq);
        real* t = a;
        a = b;
        b = t;
    }
    for (int d = 0; d < sp->ndim; ++d) {
        int e = sp->block[d];
        for (int i = 0; i < e * e; ++i) sq[i] = c->sfwd[d][i] * c->sfwd[d][i];
        apply_axis(a, b, dims, sp->ndim + 1, d + 1, sq);
        real* t = a;
        a = b;
        b = t;
    }
    if (a != out) memcpy(out, a, sizeof(real) * (size_t)total);
}

/* exact overlap-aware variance of the first kk planes
   (variance.py:758-851, :920-975): var[i,j] = sum_v V_v (sum_{e in v} E[e,(i,j)])^2 */
static void exact_variance(const stage_ctx* c, int n, int kk, const int* pos /* n x ndim abs */,
                           const real* Vvol, real* var /* kk x P */, int* cellmask_buf,
                           real* contrib) {
    const BmndStageParams* sp = c->sp;
    int ndim = sp->ndim, P = c->P;
    int minp[MAXD], ushape[MAXD], shifted[BMND_MAX_STACK][MAXD];
    for (int d = 0; d < ndim; ++d) {
        minp[d] = pos[d];
        for (int g = 1; g < n; ++g)
            if (pos[g * ndim + d] < minp[d]) minp[d] = pos[g * ndim + d];
    }
    for (int d = 0; d < ndim; ++d) {
        int mx = 0;
        for (int g = 0; g < n; ++g) {
            shifted[g][d] = pos[g * ndim + d] - minp[d];
            if (g == 0 || shifted[g][d] > mx) mx = shifted[g][d];
        }
        ushape[d] = mx + sp->block[d];
    }
    int64_t ucells = 1;
    for (int d = 0; d < ndim; ++d) ucells *= ushape[d];
    uint32_t* mask = (uint32_t*)cellmask_buf;
    memset(mask, 0, sizeof(uint32_t) * (size_t)ucells);
    for (int g = 0; g < n; ++g) {
        for (int p = 0; p < P; ++p) {
            int rem = p, loc[MAXD];
            for (int d = ndim - 1; d >= 0; --d) {
                loc[d] = rem % sp->block[d];
                rem /= sp->block[d];
            }
            int64_t cell = 0;
            for (int d = 0; d < ndim; ++d) cell = cell * ushape[d] + shifted[g][d] + loc[d];
            mask[cell] |= 1u << g;
        }
    }
    int coefs = kk * P;
    for (int i = 0; i < coefs; ++i) var[i] = 0;
    for (int64_t cell = 0; cell < ucells; ++cell) {
        uint32_t m = mask[cell];
        if (!m) continue;
        int ucoord[MAXD];
        int64_t rem = cell;
        for (int d = ndim - 1; d >= 0; --d) {
            ucoord[d] = (int)(rem % ushape[d]);
            rem /= ushape[d];
        }
        int apos[MAXD];
        for (int d = 0; d < ndim; ++d) apos[d] = ucoord[d] + minp[d];
        int64_t vidx = 0;
        for (int d = 0; d < ndim; ++d) vidx = vidx * sp->shape[d] + apos[d];
        real V = Vvol[vidx];
        for (int i = 0; i < coefs; ++i) contrib[i] = 0;
        for (int g = 0; g < n; ++g) {
            if (!(m & (1u << g))) continue;
            int p = 0;
            for (int d = 0; d < ndim; ++d) p = p * sp->block[d] + (ucoord[d] - shifted[g][d]);
            for (int i = 0; i < kk; ++i) {
                real G = c->gfwd[n][i * n + g];
                for (int j = 0; j < P; ++j) contrib[i * P + j] += G * c->S[j * P + p];
            }
        }
        for (int i = 0; i < coefs; ++i) {
            real v = contrib[i];
            var[i] = var[i] + V * v * v;
        }
    }
}

/* noise std of every coefficient (variance.py:1634-1711, :1572-1631) */
static void group_sigma(const stage_ctx* c, int n, const int* pos, const real* vgroup,
                        const real* Vvol, real* sigma, real* work, int* cellbuf) {
    const BmndStageParams* sp = c->sp;
    int P = c->P, total = n * P;
    real* approx = work;             /* total */
    real* tmp = work + total;        /* total */
    real* exact = work + 2 * total;  /* kk*P */
    real* contrib = work + 3 * total; /* kk*P */
    int k = sp->variance_k;
    if (k <= 0) {
        approx_variance(c, n, vgroup, approx, tmp);
        for (int i = 0; i < total; ++i) sigma[i] = RSQRT(approx[i] > 0 ? approx[i] : (real)0);
        return;
    }
    int kk = k < n ? k : n;
    exact_variance(c, n, kk, pos, Vvol, exact, cellbuf, contrib);
    for (int i = 0; i < kk * P; ++i) exact[i] = RSQRT(exact[i] > 0 ? exact[i] : (real)0);
    if (kk == n) {
        memcpy(sigma, exact, sizeof(real) * (size_t)total);
        return;
    }
    approx_variance(c, n, vgroup, approx, tmp);
    for (int i = 0; i < total; ++i) approx[i] = RSQRT(approx[i] > 0 ? approx[i] : (real)0);
    /* limit_poisson_group_variance_planes */
    for (int j = 0; j < P; ++j) {
        real sum_a = 0, sum_e = 0, rem_a = 0;
        for (int i = 0; i < n; ++i) {
            real s = approx[i * P + j] > 0 ? approx[i * P + j] : (real)0;
            sum_a = sum_a + s * s;
        }
        for (int i = 0; i < kk; ++i) {
            real s = exact[i * P + j] > 0 ? exact[i * P + j] : (real)0;
            sum_e = sum_e + s * s;
        }
        for (int i = kk; i < n; ++i) {
            real s = approx[i * P + j] > 0 ? approx[i * P + j] : (real)0;
            rem_a = rem_a + s * s;
        }
        real target = sum_a - sum_e;
        if (target < 0) target = 0;
        real scale = rem_a > 0 ? target / rem_a : (real)0;
        for (int i = 0; i < n; ++i) {
            real v;
            if (i < kk) {
                real s = exact[i * P + j] > 0 ? exact[i * P + j] : (real)0;
                v = s * s;
            } else {
                real s = approx[i * P + j] > 0 ? approx[i * P + j] : (real)0;
                v = s * s;
                v = v * scale;
                if (!(rem_a > 0)) v = target / (real)(n - kk);
            }
            sigma[i * P + j] = RSQRT(v > 0 ? v : (real)0);
        }
    }
}

/* poisson.py:30-46: keep iff cc > tc + 128 eps32 max(cc, tc, 1) in float64.
   *margin receives |cc - boundary| / boundary, the decision's relative
   distance from its threshold. */
static int ht_keep(real mag, real thr, double scale, double* margin) {
    double cc = (double)mag / scale;
    double tc = (double)thr / scale;
    double cs = cc > tc ? cc : tc;
    if (cs < 1.0) cs = 1.0;
    double tol = 128.0 * (double)1.1920928955078125e-07 * cs;
    double bound = tc + tol;
    *margin = bound > 0.0 ? fabs(cc - bound) / bound : INFINITY;
    return cc > bound;
}

/* aggregationweights.py:213-259, :616-630 */
static void patch_weights(const stage_ctx* c, int n, const real* att, const real* nvar,
                          real* w) {
    const BmndStageParams* sp = c->sp;
    int P = c->P;
    double plane[BMND_MAX_STACK];
    for (int g = 0; g < n; ++g) {
        double risk = 0.0;
        for (int j = 0; j < P; ++j) {
            double a = (double)att[g * P + j];
            double e = a * a;
            if (sp->weight_model != BMND_WEIGHT_CLASSIC) e *= (double)nvar[g * P + j];
            if (sp->windowed_synthesis) e *= sp->spatial_metric_diag[j];
            risk += e;
        }
        plane[g] = risk;
    }
    for (int o = 0; o < n; ++o) {
        double risk = 0.0;
        for (int g = 0; g < n; ++g) {
            double gi = (double)c->ginv[n][o * n + g];
            risk += (gi * gi) * plane[g];
        }
        if (!isfinite(risk) || risk < 0.0)
            w[o] = 0;
        else
            w[o] = (real)(1.0 / (risk + sp->eps));
    }
}

typedef struct {
    int n;
    int32_t lins[BMND_MAX_STACK];
    real weights[BMND_MAX_STACK];
    double margin; /* smallest relative distance of a hard-threshold decision from its threshold */
    real* filt;    /* n x P */
} filtered_t;

static void filter_group(const stage_ctx* c, const real* noisy, const real* pilot,
                         const real* Vvol, const int32_t* sel, int n, filtered_t* res,
                         real* buf, int* cellbuf) {
    const BmndStageParams* sp = c->sp;
    int P = c->P, ndim = sp->ndim, total = n * P;
    int pos[BMND_MAX_STACK * MAXD];
    for (int g = 0; g < n; ++g) {
        int64_t rem = sel[g];
        for (int d = ndim - 1; d >= 0; --d) {
            pos[g * ndim + d] = (int)(rem % c->counts[d]);
            rem /= c->counts[d];
        }
    }
    real* grp = buf;              /* total */
    real* coef = buf + total;     /* total */
    real* tmp = buf + 2 * total;  /* total */
    real* vg = buf + 3 * total;   /* total */
    real* sigma = buf + 4 * total; /* total */
    real* att = buf + 5 * total;  /* total */
    real* nv = buf + 6 * total;   /* total */
    real* rcoef = buf + 7 * total; /* total */
    real* work = buf + 8 * total; /* 4*total */
    for (int g = 0; g < n; ++g) {
        gather_patch(noisy, sp->shape, sp->block, ndim, pos + g * ndim, grp + g * P);
        gather_patch(Vvol, sp->shape, sp->block, ndim, pos + g * ndim, vg + g * P);
    }
    transform_group(c, n, grp, coef, tmp, 0);
    group_sigma(c, n, pos, vg, Vvol, sigma, work, cellbuf);
    for (int i = 0; i < total; ++i) nv[i] = sigma[i] * sigma[i];
    res->margin = INFINITY;
    if (sp->filter == BMND_FILTER_HARD_THRESHOLD) {
        for (int i = 0; i < total; ++i) {
            real thr = (real)sp->ht_lambda * sigma[i];
            double mg;
            int keep = ht_keep(RABS(coef[i]), thr, sp->count_scale, &mg);
            if (mg < res->margin) res->margin = mg;
            att[i] = keep ? (real)1 : (real)0;
            coef[i] = coef[i] * (keep ? (real)1 : (real)0);
        }
    } else {
        for (int g = 0; g < n; ++g)
            gather_patch(pilot, sp->shape, sp->block, ndim, pos + g * ndim, grp + g * P);
        transform_group(c, n, grp, rcoef, tmp, 0);
        for (int i = 0; i < total; ++i) {
            real eff = (real)sp->wiener_scale * nv[i];
            real pr = RABS(rcoef[i]);
            pr = pr * pr;
            real spow = pr - eff;
            if (spow < 0) spow = 0;
            real gain = spow / (spow + eff + (real)sp->eps);
            if (gain < 0) gain = 0;
            if (gain > 1) gain = 1;
            att[i] = gain;
            coef[i] = coef[i] * gain;
        }
    }
    transform_group(c, n, coef, res->filt, tmp, 1);
    patch_weights(c, n, att, nv, res->weights);
    res->n = n;
    for (int g = 0; g < n; ++g) res->lins[g] = sel[g];
}

static real* widen_volume(const float* v, int64_t nvox) {
    real* out = (real*)malloc(sizeof(real) * (size_t)nvox);
    for (int64_t i = 0; i < nvox; ++i) out[i] = (real)v[i];
    return out;
}

/*
 * One stage (bmndalgo.py:230-633 hard thresholding, :648-1046 Wiener).
 * With use_sel set, sel_io / count_io are inputs: the stage filters those
 * groups instead of matching (accepted_out is then untouched); otherwise they
 * receive the match sets when not NULL.  margin_out (n_refs doubles, or NULL)
 * receives each group's smallest relative distance of a hard-threshold
 * decision from its threshold (+inf for Wiener groups).
 */
int oracle_stage_ex(const BmndStageParams* sp, const float* noisy, const float* pilot,
                    const int32_t* refs, int64_t n_refs, float* out, int32_t* sel_io,
                    int32_t* count_io, int32_t* accepted_out, int32_t use_sel, double* margin_out,
                    int32_t threads) {
    int ndim = sp->ndim;
    stage_ctx* cp = (stage_ctx*)calloc(1, sizeof(stage_ctx));
    stage_ctx* c = cp;
    c->sp = sp;
    c->P = 1;
    int64_t nvox = 1;
    for (int d = 0; d < ndim; ++d) {
        c->P *= sp->block[d];
        c->counts[d] = sp->shape[d] - sp->block[d] + 1;
        nvox *= sp->shape[d];
    }
    int P = c->P;
    for (int n = 1; n <= sp->max_stack; ++n) {
        float f[BMND_MAX_STACK * BMND_MAX_STACK], iv[BMND_MAX_STACK * BMND_MAX_STACK];
        group_matrix(sp->group_transform, n, f, iv);
        for (int i = 0; i < n * n; ++i) {
            c->gfwd[n][i] = (real)f[i];
            c->ginv[n][i] = (real)iv[i];
        }
    }
    for (int d = 0; d < ndim; ++d)
        for (int i = 0; i < sp->block[d] * sp->block[d]; ++i) {
            c->sfwd[d][i] = (real)sp->spatial_fwd[d][i];
            c->sinv[d][i] = (real)sp->spatial_inv[d][i];
        }
    /* S = kron of spatial forwards, built axis by axis */
    c->S = (real*)malloc(sizeof(real) * (size_t)P * (size_t)P);
    {
        real* full = (real*)malloc(sizeof(real) * (size_t)P * (size_t)P);
        real* nxt = (real*)malloc(sizeof(real) * (size_t)P * (size_t)P);
        full[0] = 1;
        int fs = 1;
        for (int d = 0; d < ndim; ++d) {
            int e = sp->block[d], ns = fs * e;
            for (int i = 0; i < fs; ++i)
                for (int j = 0; j < fs; ++j)
                    for (int a = 0; a < e; ++a)
                        for (int b = 0; b < e; ++b)
                            nxt[(i * e + a) * ns + j * e + b] = full[i * fs + j] * c->sfwd[d][a * e + b];
            real* t = full;
            full = nxt;
            nxt = t;
            fs = ns;
        }
        memcpy(c->S, full, sizeof(real) * (size_t)P * (size_t)P);
        free(full);
        free(nxt);
    }
    /* variance volume (from the observation for HT, from the pilot for Wiener) */
    const float* vsrc = sp->filter == BMND_FILTER_WIENER ? pilot : noisy;
    real* Vvol = (real*)malloc(sizeof(real) * (size_t)nvox);
    for (int64_t i = 0; i < nvox; ++i) Vvol[i] = variance_value(vsrc[i], sp);
    real* noisy_r = widen_volume(noisy, nvox);
    real* pilot_r = pilot ? widen_volume(pilot, nvox) : NULL;
    int32_t* sel = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n_refs > 0 ? n_refs : 1) * (size_t)sp->max_stack);
    int32_t* cnt = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n_refs > 0 ? n_refs : 1));
    if (use_sel) {
        memcpy(sel, sel_io, sizeof(int32_t) * (size_t)n_refs * (size_t)sp->max_stack);
        memcpy(cnt, count_io, sizeof(int32_t) * (size_t)n_refs);
    } else {
        /* matching source: the observation for HT, the pilot for Wiener */
        const float* msrc = sp->filter == BMND_FILTER_WIENER ? pilot : noisy;
        BmndMatchParams mp;
        memset(&mp, 0, sizeof(mp));
        mp.ndim = ndim;
        for (int d = 0; d < ndim; ++d) {
            mp.counts[d] = c->counts[d];
            mp.search_radius[d] = sp->search_radius[d];
        }
        mp.max_matches = sp->max_stack;
        mp.min_matches = sp->min_stack;
        mp.prefer_power_of_two = 1;
        mp.distance = sp->distance;
        mp.stabilize_ties = sp->stabilize_ties;
        mp.count_scale = sp->count_scale;
        int32_t* acc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n_refs > 0 ? n_refs : 1));
        float* thr = (float*)malloc(sizeof(float) * (size_t)(n_refs > 0 ? n_refs : 1));
        for (int64_t i = 0; i < n_refs; ++i) thr[i] = sp->match_threshold;
        int32_t shape[MAXD], block[MAXD];
        for (int d = 0; d < ndim; ++d) {
            shape[d] = sp->shape[d];
            block[d] = sp->block[d];
        }
        oracle_blockmatch_volume(&mp, msrc, shape, block, refs, n_refs, thr, sel, cnt, acc, 0, threads);
        if (sel_io) memcpy(sel_io, sel, sizeof(int32_t) * (size_t)n_refs * (size_t)sp->max_stack);
        if (count_io) memcpy(count_io, cnt, sizeof(int32_t) * (size_t)n_refs);
        if (accepted_out) memcpy(accepted_out, acc, sizeof(int32_t) * (size_t)n_refs);
        free(acc);
        free(thr);
    }

    real* num = (real*)calloc((size_t)nvox, sizeof(real));
    real* den = (real*)calloc((size_t)nvox, sizeof(real));
    int64_t ushape_cap = 1;
    for (int d = 0; d < ndim; ++d) ushape_cap *= (2 * sp->search_radius[d] + sp->block[d] + 1);
    const int64_t chunk = 2048;
    filtered_t* res = (filtered_t*)malloc(sizeof(filtered_t) * (size_t)chunk);
    real* filt_store = (real*)malloc(sizeof(real) * (size_t)chunk * (size_t)sp->max_stack * (size_t)P);
    for (int64_t i = 0; i < chunk; ++i) res[i].filt = filt_store + i * sp->max_stack * P;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#endif
    for (int64_t base = 0; base < n_refs; base += chunk) {
        int64_t m = n_refs - base < chunk ? n_refs - base : chunk;
#ifdef _OPENMP
#pragma omp parallel num_threads(threads)
#endif
        {
            real* buf = (real*)malloc(sizeof(real) * (size_t)12 * (size_t)sp->max_stack * (size_t)P);
            int* cellbuf = (int*)malloc(sizeof(int) * (size_t)ushape_cap);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 8)
#endif
            for (int64_t i = 0; i < m; ++i) {
                int64_t r = base + i;
                res[i].n = 0;
                res[i].margin = INFINITY;
                if (cnt[r] <= 0) continue;
                filter_group(c, noisy_r, pilot_r, Vvol, sel + r * sp->max_stack, cnt[r], &res[i], buf,
                             cellbuf);
            }
            free(buf);
            free(cellbuf);
        }
        /* scatter in schedule order (patchaggregation.py:170-199) */
        for (int64_t i = 0; i < m; ++i) {
            if (margin_out) margin_out[base + i] = res[i].margin;
            for (int g = 0; g < res[i].n; ++g) {
                int p0[MAXD];
                int64_t rem = res[i].lins[g];
                for (int d = ndim - 1; d >= 0; --d) {
                    p0[d] = (int)(rem % c->counts[d]);
                    rem /= c->counts[d];
                }
                real w = res[i].weights[g];
                for (int p = 0; p < P; ++p) {
                    int loc[MAXD], prem = p;
                    for (int d = ndim - 1; d >= 0; --d) {
                        loc[d] = prem % sp->block[d];
                        prem /= sp->block[d];
                    }
                    int64_t x = 0;
                    for (int d = 0; d < ndim; ++d) x = x * sp->shape[d] + p0[d] + loc[d];
                    real ww = w * (real)sp->window[p];
                    num[x] = num[x] + res[i].filt[g * P + p] * ww;
                    den[x] = den[x] + ww;
                }
            }
        }
    }
    for (int64_t i = 0; i < nvox; ++i)
        out[i] = den[i] > 0 ? (float)(num[i] / (den[i] + (real)sp->eps)) : noisy[i];
    free(res);
    free(filt_store);
    free(num);
    free(den);
    free(sel);
    free(cnt);
    free(Vvol);
    free(noisy_r);
    free(pilot_r);
    free(c->S);
    free(cp);
    return BMND_OK;
}

int oracle_stage(const BmndStageParams* sp, const float* noisy, const float* pilot,
                 const int32_t* refs, int64_t n_refs, float* out, int32_t* sel_out,
                 int32_t* count_out, int32_t* accepted_out, int32_t threads) {
    return oracle_stage_ex(sp, noisy, pilot, refs, n_refs, out, sel_out, count_out, accepted_out, 0, NULL,
                           threads);
}
