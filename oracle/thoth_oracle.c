/*
 * thoth_oracle.c — TEST INFRASTRUCTURE: FP64 CPU restatement of the
 * reference's Monte-Carlo hot path (GValas/Thoth, pricer/src/...). It is the
 * parity checker for the CUDA engine and the CPU baseline timed beside it;
 * the GPU library never links or calls it.
 *
 * Every function states the reference lines whose arithmetic it restates, in
 * the same operation order so that a single-threaded run reproduces the
 * reference node graph bit for bit (pinned by tests/test_oracle_vs_reference.py
 * against the reference compiled into oracle/_ref/, and by tests/golden/): with
 * Sobol points, and with use_sobol = 0 only where a path takes one draw (the
 * reference otherwise draws in its topological schedule's order).
 * Compile with -ffp-contract=off: fused multiply-adds would change the bits.
 */
#include "thoth_oracle.h"

#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------
 * Joe-Kuo direction numbers (sobol_generator.cpp:22-76)
 * ---------------------------------------------------------------------- */
static uint32_t g_file_dims = 0;
static uint32_t* g_S = NULL;
static uint32_t* g_A = NULL;
static uint32_t* g_MOFF = NULL;
static uint32_t* g_M = NULL;

int oracle_load_direction_numbers(const char* path)
{
    FILE* f = fopen(path, "rb");
    if (!f) return -1;
    char magic[8];
    uint32_t hdr[2];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "JK621201", 8) != 0 || fread(hdr, 4, 2, f) != 2) {
        fclose(f);
        return -2;
    }
    uint32_t dims = hdr[0], nm = hdr[1];
    uint32_t* buf = (uint32_t*)malloc(sizeof(uint32_t) * (3 * (size_t)dims + 1 + nm));
    if (!buf || fread(buf, 4, 3 * (size_t)dims + 1 + nm, f) != 3 * (size_t)dims + 1 + nm) {
        free(buf);
        fclose(f);
        return -3;
    }
    fclose(f);
    free(g_S);
    g_S = buf;
    g_A = buf + dims;
    g_MOFF = buf + 2 * (size_t)dims;
    g_M = buf + 3 * (size_t)dims + 1;
    g_file_dims = dims;
    return 0;
}

static int max_dimension(void) { return (int)g_file_dims + 1; }

int oracle_direction_numbers(int dims, uint32_t* v)
{
    if (!g_S || dims < 1 || dims > max_dimension()) return -1;
    for (int i = 0; i < 32; i++) v[i] = 1u << (31 - i);
    for (int d = 1; d < dims; d++) {
        const uint32_t s = g_S[d - 1], a = g_A[d - 1];
        const uint32_t* m = g_M + g_MOFF[d - 1];
        uint32_t* V = v + 32 * (size_t)d;
        if (s >= 32) {
            for (int i = 0; i < 32; i++) V[i] = m[i] << (31 - i);
        } else {
            for (uint32_t i = 0; i < s; i++) V[i] = m[i] << (31 - i);
            for (uint32_t i = s; i < 32; i++) {
                V[i] = V[i - s] ^ (V[i - s] >> s);
                for (uint32_t k = 1; k < s; k++) V[i] ^= ((a >> (s - 1 - k)) & 1u) * V[i - k];
            }
        }
    }
    return 0;
}

/* Gray-code point n (n >= 1 is the n-th Next() after Skip): x = XOR of V[j]
 * over the set bits j of gray(n) = n ^ (n >> 1). Identical to the reference's
 * incremental Next()/Skip() (sobol_generator.cpp:80-121). */
static void sobol_point(const uint32_t* V, int dims, uint64_t n, uint32_t* x)
{
    const uint64_t g = n ^ (n >> 1);
    for (int d = 0; d < dims; d++) {
        uint32_t acc = 0;
        for (int j = 0; j < 32; j++)
            if ((g >> j) & 1u) acc ^= V[32 * (size_t)d + j];
        x[d] = acc;
    }
}

int oracle_sobol_points(int dims, int64_t skip, int64_t n, uint32_t* out)
{
    if (dims > max_dimension()) dims = max_dimension();
    uint32_t* V = (uint32_t*)malloc(sizeof(uint32_t) * 32 * (size_t)dims);
    if (!V || oracle_direction_numbers(dims, V) != 0) {
        free(V);
        return -1;
    }
    if (n > 0) sobol_point(V, dims, (uint64_t)skip + 1, out);
    for (int64_t i = 1; i < n; i++) {
        /* Gray-code increment from point skip+i to skip+i+1: flip V[ctz(skip+i+1)]... equivalently
         * the reference flips the direction number indexed by the trailing ones of skip+i */
        uint64_t c = 0;
        for (uint64_t value = (uint64_t)skip + (uint64_t)i; value & 1; value >>= 1) c++;
        for (int d = 0; d < dims; d++) out[i * dims + d] = out[(i - 1) * dims + d] ^ V[32 * (size_t)d + c];
    }
    free(V);
    return dims;
}

/* ------------------------------------------------------------------------
 * Acklam inverse normal (distributions.cpp:37-81) and Phi (:21-26)
 * ---------------------------------------------------------------------- */
double oracle_normal_cdf_inv(double P)
{
    /* Acklam's published coefficients; the same table must be used to
     * reproduce the reference's quantiles bit for bit. */
    static const double a[] = {-3.969683028665376e+01, 2.209460984245205e+02, -2.759285104469687e+02,
                               1.383577518672690e+02, -3.066479806614716e+01, 2.506628277459239e+00};
    static const double b[] = {-5.447609879822406e+01, 1.615858368580409e+02, -1.556989798598866e+02,
                               6.680131188771972e+01, -1.328068155288572e+01};
    static const double c[] = {-7.784894002430293e-03, -3.223964580411365e-01, -2.400758277161838e+00,
                               -2.549732539343734e+00, 4.374664141464968e+00, 2.938163982698783e+00};
    static const double d[] = {7.784695709041462e-03, 3.224671290700398e-01, 2.445134137142996e+00,
                               3.754408661907416e+00};
    const double p_low = 0.02425, p_high = 1.0 - p_low;
    if (P <= 0.0) return -HUGE_VAL;
    if (P >= 1.0) return HUGE_VAL;
    if (P < p_low) {
        double q = sqrt(-2.0 * log(P));
        return (((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
               ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1.0);
    }
    if (P <= p_high) {
        double q = P - 0.5;
        double r = q * q;
        return (((((a[0] * r + a[1]) * r + a[2]) * r + a[3]) * r + a[4]) * r + a[5]) * q /
               (((((b[0] * r + b[1]) * r + b[2]) * r + b[3]) * r + b[4]) * r + 1.0);
    }
    double q = sqrt(-2.0 * log(1.0 - P));
    return -(((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
           ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1.0);
}

int oracle_normal_cdf_inv_n(const double* p, int64_t n, double* out)
{
    for (int64_t i = 0; i < n; i++) out[i] = oracle_normal_cdf_inv(p[i]);
    return 0;
}

static double normal_cdf(double x) { return 0.5 * erfc(-x * M_SQRT1_2); }

/* ------------------------------------------------------------------------
 * xoshiro256++ seeded by splitmix64 (helpers/rng.hpp:36-72): tail dimensions
 * beyond the Sobol budget and use_sobol = 0.
 * ---------------------------------------------------------------------- */
typedef struct {
    uint64_t s[4];
} Xoshiro;

static uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static void xo_seed(Xoshiro* r, uint64_t seed)
{
    uint64_t z = seed;
    for (int i = 0; i < 4; i++) {
        z += 0x9e3779b97f4a7c15ULL;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
        r->s[i] = x ^ (x >> 31);
    }
}
static uint64_t xo_next(Xoshiro* r)
{
    uint64_t* s = r->s;
    const uint64_t result = rotl64(s[0] + s[3], 23) + s[0];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return result;
}
static double xo_gaussian(Xoshiro* r)
{
    const double u0 = (double)(xo_next(r) >> 11) * (1.0 / 9007199254740992.0);
    const double u = u0 > 0.0 ? u0 : (1.0 / 9007199254740992.0);
    return oracle_normal_cdf_inv(u);
}

/* ------------------------------------------------------------------------
 * Brownian bridge (path_generator.cpp:49-198)
 * ---------------------------------------------------------------------- */
typedef struct {
    int m, factors, sobol_dim;
    const double* t;       /* [m+1] */
    int *bi, *li, *ri;     /* [m] */
    double *lw, *rw, *sd;  /* [m] */
    uint32_t* V;           /* [sobol_dim][32] */
    uint32_t* x;           /* current Sobol integer point */
    uint64_t count;        /* Next() calls so far, including the skip */
    double* z;             /* [factors][m] */
    double* w;             /* [m] */
    double* noise;         /* [factors][m+1] */
    Xoshiro* rng;
} Bridge;

static int bridge_init(Bridge* B, const double* t, int n_dates, int factors, int64_t skip, int use_sobol,
                       Xoshiro* rng)
{
    memset(B, 0, sizeof *B);
    B->m = n_dates - 1;
    B->factors = factors;
    B->t = t;
    B->rng = rng;
    const int m = B->m;
    if (m <= 0) return 0;
    B->bi = (int*)calloc((size_t)m * 3, sizeof(int));
    B->li = B->bi + m;
    B->ri = B->bi + 2 * m;
    B->lw = (double*)calloc((size_t)m * 3, sizeof(double));
    B->rw = B->lw + m;
    B->sd = B->lw + 2 * m;
    int* map = (int*)calloc((size_t)m, sizeof(int));
#define BT(k) (t[(k) + 1])
    map[m - 1] = 1;
    B->bi[0] = m - 1;
    B->sd[0] = sqrt(BT(m - 1));
    B->lw[0] = B->rw[0] = 0.0;
    int j = 0;
    for (int i = 1; i < m; i++) {
        while (map[j]) j++;
        int k = j;
        while (!map[k]) k++;
        int l = j + ((k - 1 - j) >> 1);
        map[l] = i + 1;
        B->bi[i] = l;
        B->li[i] = j;
        B->ri[i] = k;
        if (j != 0) {
            B->lw[i] = (BT(k) - BT(l)) / (BT(k) - BT(j - 1));
            B->rw[i] = (BT(l) - BT(j - 1)) / (BT(k) - BT(j - 1));
            B->sd[i] = sqrt((BT(l) - BT(j - 1)) * (BT(k) - BT(l)) / (BT(k) - BT(j - 1)));
        } else {
            B->lw[i] = (BT(k) - BT(l)) / BT(k);
            B->rw[i] = BT(l) / BT(k);
            B->sd[i] = sqrt(BT(l) * (BT(k) - BT(l)) / BT(k));
        }
        j = k + 1;
        if (j >= m) j = 0;
    }
#undef BT
    free(map);
    if (use_sobol) {
        long total = (long)m * factors;
        B->sobol_dim = (int)(total < max_dimension() ? total : max_dimension());
        B->V = (uint32_t*)malloc(sizeof(uint32_t) * 32 * (size_t)B->sobol_dim);
        B->x = (uint32_t*)calloc((size_t)B->sobol_dim, sizeof(uint32_t));
        oracle_direction_numbers(B->sobol_dim, B->V);
        if (skip > 0) sobol_point(B->V, B->sobol_dim, (uint64_t)skip, B->x);
        B->count = (uint64_t)skip;
    }
    B->z = (double*)calloc((size_t)factors * m, sizeof(double));
    B->w = (double*)calloc((size_t)m, sizeof(double));
    B->noise = (double*)calloc((size_t)factors * (m + 1), sizeof(double));
    return 0;
}

static void bridge_free(Bridge* B)
{
    free(B->bi);
    free(B->lw);
    free(B->V);
    free(B->x);
    free(B->z);
    free(B->w);
    free(B->noise);
}

static void bridge_next(Bridge* B)
{
    const int m = B->m, F = B->factors;
    if (m == 0) return;
    if (B->sobol_dim > 0) {
        unsigned c = 0;
        for (uint64_t value = B->count; value & 1; value >>= 1) c++;
        for (int d = 0; d < B->sobol_dim; d++) B->x[d] ^= B->V[32 * (size_t)d + c];
        B->count++;
    }
    for (int step = 0; step < m; step++) {
        for (int f = 0; f < F; f++) {
            long dim = (long)step * F + f;
            double z;
            if (dim < B->sobol_dim) {
                double u0 = B->x[dim] * (1.0 / 4294967296.0);
                double u = fmin(1.0 - 1e-12, fmax(1e-12, u0));
                z = oracle_normal_cdf_inv(u);
            } else {
                z = xo_gaussian(B->rng);
            }
            B->z[(size_t)f * m + step] = z;
        }
    }
    for (int f = 0; f < F; f++) {
        const double* z = B->z + (size_t)f * m;
        double* w = B->w;
        w[B->bi[0]] = B->sd[0] * z[0];
        for (int i = 1; i < m; i++) {
            int li = B->li[i], ri = B->ri[i], bi = B->bi[i];
            if (li != 0)
                w[bi] = B->lw[i] * w[li - 1] + B->rw[i] * w[ri] + B->sd[i] * z[i];
            else
                w[bi] = B->rw[i] * w[ri] + B->sd[i] * z[i];
        }
        double* n = B->noise + (size_t)f * (m + 1);
        double prev = 0.0;
        for (int i = 1; i <= m; i++) {
            double wi = w[i - 1];
            double dt = B->t[i] - B->t[i - 1];
            n[i] = (dt > 0) ? (wi - prev) / sqrt(dt) : 0.0;
            prev = wi;
        }
    }
}

int oracle_bridge_increments(const double* t, int n_dates, int factors, int64_t skip, int64_t n_paths,
                             uint64_t seed, double* out)
{
    Xoshiro rng;
    xo_seed(&rng, seed);
    Bridge B;
    bridge_init(&B, t, n_dates, factors, skip, 1, &rng);
    const int N = n_dates - 1;
    for (int64_t p = 0; p < n_paths; p++) {
        bridge_next(&B);
        for (int f = 0; f < factors; f++)
            for (int i = 1; i <= N; i++) out[(p * factors + f) * N + (i - 1)] = B.noise[(size_t)f * (N + 1) + i];
    }
    bridge_free(&B);
    return 0;
}

/* ------------------------------------------------------------------------
 * Book pricing: the node graph restated per path
 * ---------------------------------------------------------------------- */
typedef struct {
    double sum, sum2, c, c2, count;
} Indicator; /* monte_carlo_node.cpp:73-96 */

static void ind_update(Indicator* ind, double x)
{
    {
        const double y = x - ind->c;
        const double t = ind->sum + y;
        ind->c = (t - ind->sum) - y;
        ind->sum = t;
    }
    {
        const double y = x * x - ind->c2;
        const double t = ind->sum2 + y;
        ind->c2 = (t - ind->sum2) - y;
        ind->sum2 = t;
    }
    ind->count += 1;
}
static double ind_value(const Indicator* ind) { return ind->sum / ind->count; }
static double ind_trust(const Indicator* ind)
{
    const double n = ind->count, sum = ind->sum;
    return sqrt((ind->sum2 - sum * sum / n) / (n - 1) / n);
}

typedef struct {
    const ThothBookDesc* d;
    int64_t skip, paths;
    double* per_path;
    int64_t n_per_path;
    Indicator book;
    Indicator* prod;
    int status;
} Job;

static double lev_lookup(const ThothAsset* A, int i, double s)
{
    /* local_volatility_node.cpp:19-47 */
    const double* v = A->lev_values + (size_t)i * A->lev_points;
    const double ln_step = A->lev_ln_step[i];
    const long offset = (long)A->lev_offset[i];
    const double f = log(s) / ln_step - (double)offset;
    const size_t last = (size_t)A->lev_points - 1;
    if (f <= 0.0) return v[0];
    if (f >= (double)last) return v[last];
    const size_t k = (size_t)f;
    const double w = f - (double)k;
    return (1.0 - w) * v[k] + w * v[k + 1];
}

static double payoff_vanilla(double s, double k, int type)
{
    /* finance.cpp:9-32 with has_cap = false, has_floor = true, floor = 0 */
    double vanilla = (type == THOTH_CALL) ? (s - k) : (k - s);
    return (vanilla < 0.0) ? 0.0 : vanilla; /* std::max(vanilla, 0.0) */
}

static void* run_job(void* arg)
{
    Job* J = (Job*)arg;
    const ThothBookDesc* d = J->d;
    const int nd = d->n_dates, N = nd - 1, na = d->n_assets;
    double* tl = (double*)malloc(sizeof(double) * nd * 3);
    double* dtl = tl + nd;
    double* sdt = tl + 2 * nd;
    /* MonteCarloNode::SetDateList (monte_carlo_node.cpp:100-124) */
    for (int i = 0; i < nd; i++) {
        tl[i] = d->days ? (double)(d->days[i] - d->days[0]) / 365.0 : d->t[i];
        if (i > 0) {
            dtl[i] = d->days ? (double)(d->days[i] - d->days[i - 1]) / 365.0 : d->t[i] - d->t[i - 1];
            sdt[i] = sqrt(dtl[i]);
        } else {
            dtl[i] = sdt[i] = 0;
        }
    }
    int F = na;
    int* vol_factor = (int*)malloc(sizeof(int) * na);
    for (int a = 0; a < na; a++) vol_factor[a] = (d->assets[a].model != THOTH_MODEL_GBM) ? F++ : -1;

    Xoshiro rng;
    xo_seed(&rng, d->seed);
    Bridge B;
    bridge_init(&B, tl, nd, F, J->skip, d->use_sobol, &rng);

    double* S = (double*)malloc(sizeof(double) * na * nd);  /* spot path per asset */
    double* V = (double*)malloc(sizeof(double) * na * nd);  /* variance path */
    double* W = (double*)malloc(sizeof(double) * na * nd);  /* Brownian (GBM) */
    double* noise = (double*)malloc(sizeof(double) * F);
    const int np = d->n_products;
    memset(&J->book, 0, sizeof J->book);
    J->prod = (Indicator*)calloc((size_t)np, sizeof(Indicator));

    for (int64_t path = 0; path < J->paths; path++) {
        if (d->use_sobol) bridge_next(&B);
        for (int a = 0; a < na; a++) {
            S[a * nd] = d->assets[a].spot;
            V[a * nd] = d->assets[a].v0;
            W[a * nd] = 0.0;
        }
        for (int i = 1; i <= N; i++) {
            /* noise nodes (noise_node.cpp:20-25). use_sobol = 0: drawn date by date in factor
             * order; the reference draws in the order of its topological schedule
             * (core/node_collector.cpp:225-340), the same stream only where a path takes one
             * draw, so that mode is compared statistically */
            for (int f = 0; f < F; f++) noise[f] = d->use_sobol ? B.noise[(size_t)f * (N + 1) + i] : xo_gaussian(&rng);
            for (int a = 0; a < na; a++) {
                const ThothAsset* A = &d->assets[a];
                const double carry_drift = A->carry[i] * tl[i] - A->carry[i - 1] * tl[i - 1];
                if (A->model == THOTH_MODEL_GBM) {
                    /* correlated noise (correlated_noise_node.cpp:15-27) */
                    double nz;
                    if (na > 1 && d->cholesky) {
                        nz = 0;
                        for (int v = 0; v < na; v++) {
                            const double l = d->cholesky[a * na + v];
                            if (l != 0) nz += noise[v] * l;
                        }
                    } else {
                        nz = noise[a];
                    }
                    /* brownian_node.cpp:12-24 */
                    W[a * nd + i] = W[a * nd + i - 1] + sdt[i] * nz;
                    /* spot_diffusion_node.cpp:21-73 (no dividends, constant vol) */
                    const double s0 = S[a * nd + i - 1] - 0;
                    const double dw = W[a * nd + i] - W[a * nd + i - 1];
                    const double v = A->vol, dt = dtl[i];
                    const double expo = carry_drift - v * v / 2 * dt + v * dw;
                    S[a * nd + i] = s0 * exp(expo) + 0;
                } else {
                    /* heston_variance_node.cpp:17-57 */
                    const double v = V[a * nd + i - 1], dt = dtl[i], z = noise[vol_factor[a]];
                    const double kappa = A->kappa, theta = A->theta, xi = A->xi;
                    const double e = exp(-kappa * dt);
                    const double m = theta + (v - theta) * e;
                    const double s2 = v * xi * xi * e / kappa * (1 - e) + theta * xi * xi / (2 * kappa) * (1 - e) * (1 - e);
                    const double psi = (m > 0) ? s2 / (m * m) : 0;
                    double vn;
                    if (psi <= 1.5) {
                        const double c = 2.0 / psi;
                        const double b2 = c - 1.0 + sqrt(c) * sqrt(c - 1.0);
                        const double aa = m / (1.0 + b2);
                        const double bz = sqrt(b2) + z;
                        vn = aa * bz * bz;
                    } else {
                        const double p = (psi - 1.0) / (psi + 1.0);
                        const double beta = (1.0 - p) / m;
                        const double u = 0.5 * erfc(-z / sqrt(2.0));
                        vn = (u <= p) ? 0.0 : log((1.0 - p) / (1.0 - u)) / beta;
                    }
                    V[a * nd + i] = vn;
                    /* heston_spot_node.cpp:32-94 */
                    const double vp = v, vc = vn, rho = A->rho;
                    /* the spot's white noise (single.cpp:88); with correlate_all_spots (an extension
                     * of this project, not the reference's behaviour) correlated through the Cholesky
                     * factor as a GBM Brownian is */
                    double zs = noise[a];
                    if (d->correlate_all_spots && na > 1 && d->cholesky) {
                        zs = 0;
                        for (int v2 = 0; v2 < na; v2++) {
                            const double l = d->cholesky[a * na + v2];
                            if (l != 0) zs += noise[v2] * l;
                        }
                    }
                    const double L = (A->model == THOTH_MODEL_LSV) ? lev_lookup(A, i, S[a * nd + i - 1]) : 1.0;
                    double step;
                    if (xi > 1e-12) {
                        const double g = 0.5;
                        const double K0 = -L * rho * kappa * theta / xi * dt;
                        const double aa = g * dt * (L * kappa * rho / xi - 0.5 * L * L);
                        const double K1 = aa - L * rho / xi;
                        const double K2 = aa + L * rho / xi;
                        const double K3 = g * dt * (1.0 - rho * rho) * L * L;
                        const double K4 = K3;
                        double var = K3 * vp + K4 * vc;
                        if (var < 0) var = 0;
                        step = carry_drift + K0 + K1 * vp + K2 * vc + sqrt(var) * zs;
                    } else {
                        step = carry_drift - 0.5 * L * L * vp * dt + L * sqrt(vp * dt) * zs;
                    }
                    S[a * nd + i] = S[a * nd + i - 1] * exp(step);
                }
            }
        }
        /* flows, contracts and the book (contract_node.cpp:16-51, book_node.cpp:16-31) */
        double book = 0;
        for (int p = 0; p < np; p++) {
            const ThothProduct* P = &d->products[p];
            const int mat = P->maturity;
#define SPOT(a, i) ((P->quanto == 0 || (i) == 0) ? S[(a) * nd + (i)] : S[(a) * nd + (i)] * exp(-P->quanto * 1.0 * 1.0 * tl[i]))
            double flow = 0;
            if (P->kind == THOTH_PRODUCT_VANILLA) {
                flow = payoff_vanilla(SPOT(P->asset, mat), P->strike, P->option_type);
            } else if (P->kind == THOTH_PRODUCT_BASKET) {
                double x = 0;
                for (int k = 0; k < P->n_components; k++) x += SPOT(P->components[k], mat) * P->weights[k];
                flow = payoff_vanilla(x, P->strike, P->option_type);
            } else if (P->kind == THOTH_PRODUCT_BARRIER) {
                int hit = 0;
                for (int k = 0; k < P->n_monitor; k++) {
                    const double s = SPOT(P->asset, P->monitor[k]);
                    if (P->barrier_up ? (s >= P->barrier_level) : (s <= P->barrier_level)) {
                        hit = 1;
                        break;
                    }
                }
                const int alive = P->barrier_in ? hit : !hit;
                flow = alive ? payoff_vanilla(SPOT(P->asset, mat), P->strike, P->option_type) : 0;
            } else if (P->kind == THOTH_PRODUCT_VARIANCE) {
                double sum2 = 0, prev = SPOT(P->asset, 0);
                if (P->n_obs == 0) {
                    for (int j = 1; j <= mat; j++) {
                        const double s = SPOT(P->asset, j);
                        const double r = log(s / prev);
                        sum2 += r * r;
                        prev = s;
                    }
                } else {
                    for (int k = 0; k < P->n_obs; k++) {
                        const double s = SPOT(P->asset, P->obs[k]);
                        const double r = log(s / prev);
                        sum2 += r * r;
                        prev = s;
                    }
                }
                const double T = (P->total_year_fraction > 0) ? P->total_year_fraction : tl[mat];
                const double rv = (T > 0) ? (P->past_variance + sum2) / T : 0;
                flow = P->notional * (rv - P->strike_variance);
            }
#undef SPOT
            double df = 1;
            if (mat != 0) {
                const double dt1 = tl[0], dt2 = tl[mat];
                df = exp(dt1 * P->zero_rate - dt2 * P->zero_rate);
            }
            const double x = 0 + flow * df;
            ind_update(&J->prod[p], x);
            if (J->per_path && path < J->n_per_path) J->per_path[path * np + p] = x;
            book += x * P->fx;
        }
        ind_update(&J->book, book);
    }
    bridge_free(&B);
    free(S);
    free(V);
    free(W);
    free(noise);
    free(vol_factor);
    free(tl);
    J->status = 0;
    return NULL;
}

int oracle_price_book(const ThothBookDesc* d, ThothBookResult* r, int threads, double* per_path, int64_t n_per_path)
{
    if (!d || !r || d->n_dates < 2 || d->paths < 2 || d->n_assets < 1) return THOTH_GPU_E_INVALID;
    if (d->use_sobol && !g_S) return THOTH_GPU_E_INVALID;
    if (threads < 1) threads = 1;
    if (threads > d->paths / 2) threads = (int)(d->paths / 2);
    Job* jobs = (Job*)calloc((size_t)threads, sizeof(Job));
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    int64_t done = 0;
    for (int k = 0; k < threads; k++) {
        /* balanced split, skip = running count (run_cluster.cpp:308-340) */
        const int64_t n = d->paths / threads + (k < d->paths % threads ? 1 : 0);
        jobs[k].d = d;
        jobs[k].skip = d->sobol_skip + done;
        jobs[k].paths = n;
        jobs[k].per_path = (k == 0) ? per_path : NULL;
        jobs[k].n_per_path = n_per_path;
        done += n;
    }
    if (threads == 1) {
        run_job(&jobs[0]);
    } else {
        for (int k = 0; k < threads; k++) pthread_create(&th[k], NULL, run_job, &jobs[k]);
        for (int k = 0; k < threads; k++) pthread_join(th[k], NULL);
    }
    /* pooling: value = sum w_k v_k, trust^2 = sum w_k^2 trust_k^2 (run_cluster.cpp:413-445) */
    const double total = (double)d->paths;
    double bv = 0, bt2 = 0;
    for (int k = 0; k < threads; k++) {
        const double w = (double)jobs[k].paths / total;
        bv += w * ind_value(&jobs[k].book);
        const double t = ind_trust(&jobs[k].book);
        bt2 += w * w * t * t;
    }
    r->book_premium = bv;
    r->book_trust = sqrt(bt2);
    for (int p = 0; p < d->n_products; p++) {
        double v = 0, t2 = 0;
        for (int k = 0; k < threads; k++) {
            const double w = (double)jobs[k].paths / total;
            v += w * ind_value(&jobs[k].prod[p]);
            const double t = ind_trust(&jobs[k].prod[p]);
            t2 += w * w * t * t;
        }
        if (r->premium) r->premium[p] = v;
        if (r->trust) r->trust[p] = sqrt(t2);
    }
    for (int k = 0; k < threads; k++) free(jobs[k].prod);
    free(jobs);
    free(th);
    r->device_ms = 0;
    return THOTH_GPU_OK;
}

/* ------------------------------------------------------------------------
 * Closed forms
 * ---------------------------------------------------------------------- */
double oracle_bs_price(double F, double K, double T, double vol, double df, int is_call)
{
    /* finance.cpp:64-85, put by parity */
    double call;
    if (vol <= 0 || T == 0 || K <= 0 || F <= 0) {
        call = df * fmax(F - K, 0.0);
    } else {
        const double v = vol * sqrt(T);
        const double d1 = log(F / K) / v + 0.5 * v;
        const double d2 = d1 - v;
        call = df * (F * normal_cdf(d1) - K * normal_cdf(d2));
    }
    return is_call ? call : call - df * (F - K);
}

double oracle_bs_delta(double S, double K, double T, double vol, double r, double q, int is_call)
{
    const double F = S * exp((r - q) * T);
    const double v = vol * sqrt(T);
    const double d1 = log(F / K) / v + 0.5 * v;
    const double e = exp(-q * T);
    return is_call ? e * normal_cdf(d1) : e * (normal_cdf(d1) - 1.0);
}

double oracle_bs_vega(double S, double K, double T, double vol, double r, double q)
{
    const double F = S * exp((r - q) * T);
    const double v = vol * sqrt(T);
    const double d1 = log(F / K) / v + 0.5 * v;
    return S * exp(-q * T) * sqrt(T) * exp(-0.5 * d1 * d1) / sqrt(2.0 * M_PI);
}

/* Heston P_j integrand in the "little Heston trap" form (Albrecher et al.
 * 2007), forward measure: the formulation of finance.cpp:472-513. */
typedef struct {
    double F, K, T, v0, kappa, theta, xi, rho;
    int j;
} HestonP;

static double heston_integrand(double phi, const HestonP* h)
{
    const double complex IU = _Complex_I;
    const double uj = (h->j == 1) ? 0.5 : -0.5;
    const double bj = (h->j == 1) ? (h->kappa - h->rho * h->xi) : h->kappa;
    const double a = h->kappa * h->theta, xi2 = h->xi * h->xi;
    const double complex rxi = h->rho * h->xi * IU * phi;
    const double complex d = csqrt((rxi - bj) * (rxi - bj) - xi2 * (2.0 * uj * IU * phi - phi * phi));
    const double complex g = (bj - rxi - d) / (bj - rxi + d);
    const double complex edt = cexp(-d * h->T);
    const double complex C = (a / xi2) * ((bj - rxi - d) * h->T - 2.0 * clog((1.0 - g * edt) / (1.0 - g)));
    const double complex D = (bj - rxi - d) / xi2 * ((1.0 - edt) / (1.0 - g * edt));
    const double complex f = cexp(C + D * h->v0 + IU * phi * log(h->F));
    return creal(cexp(-IU * phi * log(h->K)) * f / (IU * phi));
}

/* adaptive Gauss-Kronrod 7-15 on [a, b] of g(x) = integrand(x / (1 - x)) / (1 - x)^2,
 * the map of [0, inf) onto [0, 1) */
static const double GK_X[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                               0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                               0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                               0.207784955007898467600689403773245, 0.000000000000000000000000000000000};
static const double GK_WK[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                                0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                                0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                                0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
static const double GK_WG[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                                0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

static double mapped(double x, const HestonP* h)
{
    const double om = 1.0 - x;
    return heston_integrand(x / om, h) / (om * om);
}

static double gk15(double a, double b, const HestonP* h, double* err)
{
    const double c = 0.5 * (a + b), hl = 0.5 * (b - a);
    const double fc = mapped(c, h);
    double rk = fc * GK_WK[7], rg = fc * GK_WG[3];
    for (int k = 0; k < 7; k++) {
        const double dx = hl * GK_X[k];
        const double f1 = mapped(c - dx, h), f2 = mapped(c + dx, h);
        rk += GK_WK[k] * (f1 + f2);
        if (k % 2 == 1) rg += GK_WG[k / 2] * (f1 + f2);
    }
    *err = fabs((rk - rg) * hl);
    return rk * hl;
}

static double gk_adapt(double a, double b, const HestonP* h, double tol, int depth)
{
    double err;
    const double v = gk15(a, b, h, &err);
    if (depth <= 0 || err <= tol || err <= 4e-16 * fabs(v)) return v;
    const double m = 0.5 * (a + b);
    return gk_adapt(a, m, h, 0.5 * tol, depth - 1) + gk_adapt(m, b, h, 0.5 * tol, depth - 1);
}

static double heston_prob(HestonP h, int j)
{
    h.j = j;
    /* lower bound 1e-8 as finance.cpp:524; upper end of the map stops short of 1 */
    const double a = 1e-8 / (1.0 + 1e-8);
    double total = 0;
    /* split [a, 1) into panels so that the oscillatory region is resolved */
    const double edges[] = {a, 0.02, 0.05, 0.1, 0.2, 0.35, 0.5, 0.65, 0.8, 0.9, 0.95, 0.98, 0.995, 0.9995, 1.0 - 1e-9};
    for (size_t k = 0; k + 1 < sizeof edges / sizeof edges[0]; k++) total += gk_adapt(edges[k], edges[k + 1], &h, 1e-13, 18);
    return 0.5 + total / M_PI;
}

/* Lewis (2000) single-integral form, the primary FP64 Heston oracle:
 *   C = df (F - sqrt(F K) / pi * int_0^inf Re[e^{i u k} phi(u - i/2)] / (u^2 + 1/4) du),  k = ln(F/K),
 * phi the little-trap characteristic function of ln(S_T / F). Integrated by
 * adaptive Gauss-Kronrod 7-15 on dyadic panels [0,1], [1,2], [2,4], ... until a
 * panel contributes below 1e-17; agrees with 30-digit quadrature to ~1e-12. */
typedef struct {
    double k, T, v0, kappa, theta, xi, rho;
} LewisP;

static double lewis_integrand(double u, const LewisP* h)
{
    const double complex I1 = _Complex_I;
    const double complex w = u - 0.5 * I1; /* phi(u - i/2) */
    const double xi = h->xi, rho = h->rho, kappa = h->kappa;
    const double complex b = kappa - rho * xi * I1 * w;
    const double complex d = csqrt(b * b + xi * xi * (I1 * w + w * w));
    const double complex g = (b - d) / (b + d);
    const double complex e = cexp(-d * h->T);
    const double complex C = kappa * h->theta / (xi * xi) * ((b - d) * h->T - 2.0 * clog((1.0 - g * e) / (1.0 - g)));
    const double complex D = (b - d) / (xi * xi) * (1.0 - e) / (1.0 - g * e);
    const double complex phi = cexp(C + D * h->v0);
    return creal(cexp(I1 * u * h->k) * phi) / (u * u + 0.25);
}

static double lewis_gk(double a, double b, const LewisP* h, double* err)
{
    const double c = 0.5 * (a + b), hl = 0.5 * (b - a);
    const double fc = lewis_integrand(c, h);
    double rk = fc * GK_WK[7], rg = fc * GK_WG[3];
    for (int k = 0; k < 7; k++) {
        const double dx = hl * GK_X[k];
        const double f1 = lewis_integrand(c - dx, h), f2 = lewis_integrand(c + dx, h);
        rk += GK_WK[k] * (f1 + f2);
        if (k % 2 == 1) rg += GK_WG[k / 2] * (f1 + f2);
    }
    *err = fabs((rk - rg) * hl);
    return rk * hl;
}

static double lewis_adapt(double a, double b, const LewisP* h, double tol, int depth)
{
    double err;
    const double v = lewis_gk(a, b, h, &err);
    /* absolute tolerance, floored at the rounding level of the panel value */
    if (depth <= 0 || err <= tol || err <= 4e-16 * fabs(v)) return v;
    const double m = 0.5 * (a + b);
    return lewis_adapt(a, m, h, 0.5 * tol, depth - 1) + lewis_adapt(m, b, h, 0.5 * tol, depth - 1);
}

double oracle_heston_price(double S, double K, double T, double r, double q, double v0, double kappa, double theta,
                           double xi, double rho, int is_call)
{
    const double F = S * exp((r - q) * T), df = exp(-r * T);
    double call;
    if (xi <= 1e-10 || T <= 0) {
        call = oracle_bs_price(F, K, T, sqrt(fmax(v0, 0.0)), df, 1);
    } else {
        LewisP h = {log(F / K), T, v0, kappa, theta, xi, rho};
        double total = lewis_adapt(0.0, 1.0, &h, 1e-16, 18);
        for (double a = 1.0; a < 1e7; a *= 2.0) {
            const double part = lewis_adapt(a, 2.0 * a, &h, 1e-16, 14);
            total += part;
            /* the integrand decays monotonically past its oscillations: stop once a
             * dyadic panel adds less than 1e-16 of the total (or in absolute terms) */
            if (a > 64 && (fabs(part) < 1e-17 || fabs(part) < 1e-16 * fabs(total))) break;
        }
        call = df * (F - sqrt(F * K) / M_PI * total);
    }
    return is_call ? call : call - df * (F - K);
}

/* The reference's own decomposition C = df (F P1 - K P2) (finance.cpp:541-568),
 * kept as the second rule the Lewis oracle is cross-checked against. */
double oracle_heston_price_p12(double S, double K, double T, double r, double q, double v0, double kappa,
                               double theta, double xi, double rho, int is_call)
{
    const double F = S * exp((r - q) * T), df = exp(-r * T);
    HestonP h = {F, K, T, v0, kappa, theta, xi, rho, 1};
    const double call = df * (F * heston_prob(h, 1) - K * heston_prob(h, 2));
    return is_call ? call : call - df * (F - K);
}

/* many Heston prices at once on `threads` host threads; args[i] = (S, K, T, r, q,
 * v0, kappa, theta, xi, rho), calls. */
typedef struct {
    const double* args;
    double* out;
    int64_t lo, hi;
} CfJob;

static void* cf_job(void* p)
{
    CfJob* j = (CfJob*)p;
    for (int64_t i = j->lo; i < j->hi; i++) {
        const double* a = j->args + 10 * i;
        j->out[i] = oracle_heston_price(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], 1);
    }
    return NULL;
}

int oracle_heston_prices(int64_t n, const double* args, double* out, int threads)
{
    if (threads < 1) threads = 1;
    pthread_t th[256];
    CfJob jobs[256];
    if (threads > 256) threads = 256;
    for (int k = 0; k < threads; k++) {
        jobs[k].args = args;
        jobs[k].out = out;
        jobs[k].lo = n * k / threads;
        jobs[k].hi = n * (k + 1) / threads;
        pthread_create(&th[k], NULL, cf_job, &jobs[k]);
    }
    for (int k = 0; k < threads; k++) pthread_join(th[k], NULL);
    return 0;
}


/* ------------------------------------------------------------------------
 * LSV leverage calibration: Single::CalibrateLeverage and its helpers
 * (marketdata/single.cpp:240-473) in the same operation order.
 * ---------------------------------------------------------------------- */
int oracle_xoshiro_draws(uint64_t seed, uint64_t skip, int64_t n, uint64_t* out, uint64_t state_out[4])
{
    Xoshiro r;
    xo_seed(&r, seed);
    for (uint64_t i = 0; i < skip; i++) xo_next(&r);
    for (int64_t i = 0; i < n; i++) out[i] = xo_next(&r);
    if (state_out) memcpy(state_out, r.s, sizeof r.s);
    return 0;
}

typedef struct {
    double x0, dx, fallback;
    int n;
    double* mean;
} CondVar;

/* binned E[v | ln S] (single.cpp:256-316): equal-width bins between the extremes,
 * thin bins from the nearest populated neighbour (left first), the ensemble mean
 * while the extremes coincide */
static void condvar_build(CondVar* cv, const double* ln, const double* var, int P, int bins, int min_count,
                          double* sum, int* count)
{
    double fb = 0;
    for (int p = 0; p < P; p++) fb += var[p];
    fb /= (double)P;
    cv->fallback = fb;
    cv->n = 0;
    double mn = ln[0], mx = ln[0];
    for (int p = 1; p < P; p++) {
        if (ln[p] < mn) mn = ln[p];
        if (ln[p] > mx) mx = ln[p];
    }
    if (mx - mn < 1e-10) return;
    const double width = (mx - mn) / bins;
    for (int b = 0; b < bins; b++) {
        sum[b] = 0.0;
        count[b] = 0;
    }
    for (int p = 0; p < P; p++) {
        int b = (int)((ln[p] - mn) / width);
        b = b < 0 ? 0 : (b > bins - 1 ? bins - 1 : b);
        sum[b] += var[p];
        count[b]++;
    }
    for (int b = 0; b < bins; b++) cv->mean[b] = fb;
    for (int b = 0; b < bins; b++)
        if (count[b] >= min_count) cv->mean[b] = sum[b] / count[b];
    for (int b = 0; b < bins; b++) {
        if (count[b] >= min_count) continue;
        for (int d = 1; d < bins; d++) {
            if (b - d >= 0 && count[b - d] >= min_count) {
                cv->mean[b] = sum[b - d] / count[b - d];
                break;
            }
            if (b + d < bins && count[b + d] >= min_count) {
                cv->mean[b] = sum[b + d] / count[b + d];
                break;
            }
        }
    }
    cv->x0 = mn + 0.5 * width;
    cv->dx = width;
    cv->n = bins;
}

static double condvar_at(const CondVar* cv, double X)
{
    if (cv->n == 0) return cv->fallback;
    const double f = (X - cv->x0) / cv->dx;
    const double last = (double)(cv->n - 1);
    if (f <= 0) return cv->mean[0];
    if (f >= last) return cv->mean[cv->n - 1];
    const size_t i = (size_t)f;
    const double w = f - (double)i;
    return (1.0 - w) * cv->mean[i] + w * cv->mean[i + 1];
}

/* one Andersen QE variance step (single.cpp:344-368) */
static double calib_qe(double V, double Dt, double Z, double kappa, double theta, double xi)
{
    const double e = exp(-kappa * Dt);
    const double m = theta + (V - theta) * e;
    const double s2 = V * xi * xi * e / kappa * (1 - e) + theta * xi * xi / (2 * kappa) * (1 - e) * (1 - e);
    const double psi = (m > 0) ? s2 / (m * m) : 0;
    if (psi <= 1.5) {
        const double c = 2.0 / psi;
        const double b2 = c - 1.0 + sqrt(c) * sqrt(c - 1.0);
        const double a = m / (1.0 + b2);
        const double bz = sqrt(b2) + Z;
        return a * bz * bz;
    }
    const double p = (psi - 1.0) / (psi + 1.0);
    const double beta = (1.0 - p) / m;
    const double u = 0.5 * erfc(-Z / sqrt(2.0));
    return (u <= p) ? 0.0 : log((1.0 - p) / (1.0 - u)) / beta;
}

/* one leveraged Andersen log-spot step (single.cpp:370-388) */
static double calib_spot(double Vp, double Vc, double Dt, double Carry, double L, double Z, double kappa,
                         double theta, double xi, double rho)
{
    if (xi > 1e-12) {
        const double g = 0.5;
        const double k0 = -L * rho * kappa * theta / xi * Dt;
        const double a = g * Dt * (L * kappa * rho / xi - 0.5 * L * L);
        const double k1 = a - L * rho / xi;
        const double k2 = a + L * rho / xi;
        const double k3 = g * Dt * (1.0 - rho * rho) * L * L;
        double var = k3 * (Vp + Vc);
        if (var < 0) var = 0;
        return Carry + k0 + k1 * Vp + k2 * Vc + sqrt(var) * Z;
    }
    return Carry - 0.5 * L * L * Vp * Dt + L * sqrt(Vp * Dt) * Z;
}

/* LeverageSurface::LayerAt (leverage_surface.cpp:19-40) */
static double layer_at(const double* lev, int points, double ln_step, int64_t offset, double S)
{
    const double f = log(S) / ln_step - (double)offset;
    const int last = points - 1;
    if (!(f > 0.0)) return lev[0];
    if (f >= (double)last) return lev[last];
    const size_t i = (size_t)f;
    const double w = f - (double)i;
    return (1.0 - w) * lev[i] + w * lev[i + 1];
}

int oracle_calibrate_leverage(ThothLeverageCalib* c)
{
    const int P = c->particles > 0 ? c->particles : 16384;
    const int bins = c->bins > 0 ? c->bins : 30;
    const int min_count = c->min_bin_count > 0 ? c->min_bin_count : 20;
    const double min_cv = c->min_cond_variance > 0 ? c->min_cond_variance : 1e-6;
    const double lmin = c->lev_min > 0 ? c->lev_min : 0.05, lmax = c->lev_max > 0 ? c->lev_max : 10.0;
    const int n = c->n_dates, pts = c->points;
    if (n < 1 || pts < 2 || !c->days || !c->carry || !c->ln_step || !c->offset || !c->local_vol || !c->leverage)
        return -1;
    double* spot = malloc(sizeof(double) * P);
    double* var = malloc(sizeof(double) * P);
    double* ln = malloc(sizeof(double) * P);
    double* mean = malloc(sizeof(double) * bins);
    double* sum = malloc(sizeof(double) * bins);
    int* count = malloc(sizeof(int) * bins);
    Xoshiro rng;
    xo_seed(&rng, c->seed);
    for (int p = 0; p < P; p++) {
        spot[p] = c->spot;
        var[p] = c->v0;
        ln[p] = log(c->spot);
    }
    CondVar cv = {0, 1, 0, 0, mean};
    for (int k = 0; k < n; k++) {
        condvar_build(&cv, ln, var, P, bins, min_count, sum, count);
        double* layer = c->leverage + (size_t)k * pts;
        for (int i = 0; i < pts; i++) {
            const double x = (double)(c->offset[k] + i) * c->ln_step[k];
            const double sig = c->local_vol[(size_t)k * pts + i];
            double ev = condvar_at(&cv, x);
            if (ev < min_cv) ev = min_cv;
            double L = sig / sqrt(ev);
            layer[i] = L < lmin ? lmin : (L > lmax ? lmax : L);
        }
        if (k == 0) continue;
        const double dt = (double)(c->days[k] - c->days[k - 1]) / 365.0;
        const double carry = c->carry[k] * ((double)c->days[k] / 365.0) - c->carry[k - 1] * ((double)c->days[k - 1] / 365.0);
        for (int p = 0; p < P; p++) {
            const double lp = layer_at(layer, pts, c->ln_step[k], c->offset[k], spot[p]);
            const double vp = var[p];
            const double vc = calib_qe(vp, dt, xo_gaussian(&rng), c->kappa, c->theta, c->xi);
            const double step = calib_spot(vp, vc, dt, carry, lp, xo_gaussian(&rng), c->kappa, c->theta, c->xi, c->rho);
            var[p] = vc;
            spot[p] *= exp(step);
            ln[p] += step;
        }
    }
    free(spot);
    free(var);
    free(ln);
    free(mean);
    free(sum);
    free(count);
    return 0;
}
