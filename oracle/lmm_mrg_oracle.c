/*
 * lmm_mrg_oracle.c -- TEST INFRASTRUCTURE ONLY. This is the checker, never the
 * product: only tests/ and bench.py's CPU legs load it.
 *
 * CPU restatement of the normal stream that the reference draws in
 * LiborMarketModel/mklRng.cpp:44-110: ONE MRG32k3a stream seeded with 12345
 * (vslNewStream(&stream, VSL_BRNG_MRG32K3A, seed), :91, default seed in
 * mklRng.h), read sequentially into z[0..num) -- each OpenMP thread skips
 * ahead to its first element (vslSkipAheadStream, :97) -- with Gaussians by
 * inversion (VSL_RNG_METHOD_GAUSSIAN_ICDF, :25/:31), z = mean + stddev * x.
 * MKL is closed and absent here; this file restates the published algorithms:
 *
 *   MRG32k3a  P. L'Ecuyer, "Good parameters and implementations for combined
 *             multiple recursive random number generators", Operations
 *             Research 47(1):159-164, 1999. Two order-3 recurrences
 *               x_n = (1403580 x_{n-2} - 810728 x_{n-3}) mod m1,  m1 = 2^32 - 209
 *               y_n = (527612 y_{n-1} - 1370589 y_{n-3}) mod m2,  m2 = 2^32 - 22853
 *             combined as z_n = (x_n - y_n) mod m1 in [1, m1] (0 maps to m1)
 *             and u_n = z_n / (m1 + 1), the paper's normalisation.
 *   skip-ahead  the state (x_{n-3}, x_{n-2}, x_{n-1}) advances by the 3x3
 *             companion matrix A1 (A2 for y); element e is produced from
 *             A^e s_0, with A^e assembled from A^(2^k) (L'Ecuyer, Simard,
 *             Chen, Kelton, Operations Research 50(6), 2002, which also lists
 *             A1^(2^76), A2^(2^76), A1^(2^127), A2^(2^127): the tests pin the
 *             matrix powers here against those published values).
 *   seeding   one 32-bit seed s: x state (s mod m1, 1, 1), y state (1, 1, 1)
 *             (a zero x state is replaced by (1, 1, 1)). This is this
 *             library's convention; MKL's exact seeding and output scaling
 *             are not documented here, so parity with MKL's numbers is
 *             UNPINNED -- only the generator family, its stream order and
 *             the inversion method follow the reference.
 *   inversion M. J. Wichura, "Algorithm AS 241: The percentage points of the
 *             normal distribution", Applied Statistics 37(3):477-484, 1988:
 *             PPND16 (relative error about 1e-16) for FP64 output, PPND7
 *             (about 1e-7) evaluated in FP32 for FP32 output.
 */
#include <math.h>
#include <stdint.h>

#define M1 4294967087ULL
#define M2 4294944443ULL

typedef struct { uint64_t a[9]; } mat3;

static const mat3 A1 = {{0, 1, 0, 0, 0, 1, M1 - 810728ULL, 1403580ULL, 0}};
static const mat3 A2 = {{0, 1, 0, 0, 0, 1, M2 - 1370589ULL, 0, 527612ULL}};

static uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (a * b) % m; }

static mat3 matmul(const mat3 *x, const mat3 *y, uint64_t m)
{
    mat3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            uint64_t s = 0;
            for (int k = 0; k < 3; ++k) s = (s + mulmod(x->a[3 * i + k], y->a[3 * k + j], m)) % m;
            r.a[3 * i + j] = s;
        }
    return r;
}

static void matvec(const mat3 *x, uint64_t v[3], uint64_t m)
{
    uint64_t r[3];
    for (int i = 0; i < 3; ++i) {
        uint64_t s = 0;
        for (int k = 0; k < 3; ++k) s = (s + mulmod(x->a[3 * i + k], v[k], m)) % m;
        r[i] = s;
    }
    v[0] = r[0];
    v[1] = r[1];
    v[2] = r[2];
}

static mat3 matpow(mat3 a, uint64_t e, uint64_t m)
{
    mat3 r = {{1, 0, 0, 0, 1, 0, 0, 0, 1}};
    /* e is a 64-bit count; powers 2^76 and 2^127 are reached by squaring */
    while (e) {
        if (e & 1) r = matmul(&r, &a, m);
        a = matmul(&a, &a, m);
        e >>= 1;
    }
    return r;
}

/* A1^(2^k) and A2^(2^k) for the published-value pins (k up to 127). */
void lmmo_mrg32k3a_pow2(int32_t k, uint64_t a1[9], uint64_t a2[9])
{
    mat3 x = A1, y = A2;
    for (int i = 0; i < k; ++i) {
        x = matmul(&x, &x, M1);
        y = matmul(&y, &y, M2);
    }
    for (int i = 0; i < 9; ++i) {
        a1[i] = x.a[i];
        a2[i] = y.a[i];
    }
}

static void seed_state(uint32_t seed, uint64_t x[3], uint64_t y[3])
{
    x[0] = seed % M1;
    x[1] = 1;
    x[2] = 1;
    y[0] = y[1] = y[2] = 1;
}

/* One step of both recurrences; returns z in [1, m1]. */
static uint32_t next_z(uint64_t x[3], uint64_t y[3])
{
    /* each product is below 2^53, so the differences fit in int64 */
    int64_t p1 = ((int64_t)(1403580ULL * x[1]) - (int64_t)(810728ULL * x[0])) % (int64_t)M1;
    int64_t p2 = ((int64_t)(527612ULL * y[2]) - (int64_t)(1370589ULL * y[0])) % (int64_t)M2;
    if (p1 < 0) p1 += (int64_t)M1;
    if (p2 < 0) p2 += (int64_t)M2;
    x[0] = x[1];
    x[1] = x[2];
    x[2] = (uint64_t)p1;
    y[0] = y[1];
    y[1] = y[2];
    y[2] = (uint64_t)p2;
    return (uint32_t)(p1 > p2 ? p1 - p2 : p1 - p2 + (int64_t)M1);
}

static double next_u(uint64_t x[3], uint64_t y[3]) { return (double)next_z(x, y) * (1.0 / 4294967088.0); }

/* Sequential stream elements [first, first+count) as uniforms in (0,1). */
void lmmo_mrg32k3a_uniforms(uint32_t seed, int64_t first, int64_t count, double *u)
{
    uint64_t x[3], y[3];
    seed_state(seed, x, y);
    mat3 p1 = matpow(A1, (uint64_t)first, M1), p2 = matpow(A2, (uint64_t)first, M2);
    matvec(&p1, x, M1);
    matvec(&p2, y, M2);
    for (int64_t i = 0; i < count; ++i) u[i] = next_u(x, y);
}

static double poly(const double *c, int n, double x)
{
    double r = c[n - 1];
    for (int i = n - 2; i >= 0; --i) r = r * x + c[i];
    return r;
}

/* AS241 PPND16. */
double lmmo_ppnd16(double p)
{
    static const double a[8] = {3.3871328727963666080e0, 1.3314166789178437745e+2,
                                1.9715909503065514427e+3, 1.3731693765509461125e+4,
                                4.5921953931549871457e+4, 6.7265770927008700853e+4,
                                3.3430575583588128105e+4, 2.5090809287301226727e+3};
    static const double b[8] = {1.0, 4.2313330701600911252e+1, 6.8718700749205790830e+2,
                                5.3941960214247511077e+3, 2.1213794301586595867e+4,
                                3.9307895800092710610e+4, 2.8729085735721942674e+4,
                                5.2264952788528545610e+3};
    static const double c[8] = {1.42343711074968357734e0, 4.63033784615654529590e0,
                                5.76949722146069140550e0, 3.64784832476320460504e0,
                                1.27045825245236838258e0, 2.41780725177450611770e-1,
                                2.27238449892691845833e-2, 7.74545014278341407640e-4};
    static const double d[8] = {1.0, 2.05319162663775882187e0, 1.67638483018380384940e0,
                                6.89767334985100004550e-1, 1.48103976427480074590e-1,
                                1.51986665636164571966e-2, 5.47593808499534494600e-4,
                                1.05075007164441684324e-9};
    static const double e[8] = {6.65790464350110377720e0, 5.46378491116411436990e0,
                                1.78482653991729133580e0, 2.96560571828504891230e-1,
                                2.65321895265761230930e-2, 1.24266094738807843860e-3,
                                2.71155556874348757815e-5, 2.01033439929228813265e-7};
    static const double f[8] = {1.0, 5.99832206555887937690e-1, 1.36929880922735805310e-1,
                                1.48753612908506148525e-2, 7.86869131145613259100e-4,
                                1.84631831751005468180e-5, 1.42151175831644588870e-7,
                                2.04426310338993978564e-15};
    const double q = p - 0.5;
    if (fabs(q) <= 0.425) {
        const double r = 0.180625 - q * q;
        return q * poly(a, 8, r) / poly(b, 8, r);
    }
    double r = q < 0.0 ? p : 1.0 - p;
    r = sqrt(-log(r));
    double v;
    if (r <= 5.0) {
        r -= 1.6;
        v = poly(c, 8, r) / poly(d, 8, r);
    } else {
        r -= 5.0;
        v = poly(e, 8, r) / poly(f, 8, r);
    }
    return q < 0.0 ? -v : v;
}

/* AS241 PPND7 in FP32 arithmetic. The caller passes q = p - 1/2 and the
 * smaller tail probability pt = min(p, 1-p), both formed from the integer
 * stream value, so that no FP32 cancellation near p = 1 occurs. */
float lmmo_ppnd7(float q, float pt)
{
    if (fabsf(q) <= 0.425f) {
        const float r = 0.180625f - q * q;
        return q * (((59.109374720f * r + 159.29113202f) * r + 50.434271938f) * r + 3.3871327179f) /
               (((67.187563600f * r + 78.757757664f) * r + 17.895169469f) * r + 1.0f);
    }
    float r = sqrtf(-logf(pt));
    float v;
    if (r <= 5.0f) {
        r -= 1.6f;
        v = (((0.17023821103f * r + 1.3067284816f) * r + 2.7568153900f) * r + 1.4234372777f) /
            ((0.12021132975f * r + 0.73700164250f) * r + 1.0f);
    } else {
        r -= 5.0f;
        v = (((0.017337203997f * r + 0.42868294337f) * r + 3.0812263860f) * r + 6.6579051150f) /
            ((0.012258202635f * r + 0.24197894225f) * r + 1.0f);
    }
    return q < 0.0f ? -v : v;
}

void lmmo_mrg32k3a_normals_f64(uint32_t seed, int64_t first, int64_t count, double mean, double sd,
                               double *z)
{
    lmmo_mrg32k3a_uniforms(seed, first, count, z);
    for (int64_t i = 0; i < count; ++i) z[i] = mean + sd * lmmo_ppnd16(z[i]);
}

void lmmo_mrg32k3a_normals_f32(uint32_t seed, int64_t first, int64_t count, float mean, float sd,
                               float *z)
{
    uint64_t x[3], y[3];
    seed_state(seed, x, y);
    mat3 p1 = matpow(A1, (uint64_t)first, M1), p2 = matpow(A2, (uint64_t)first, M2);
    matvec(&p1, x, M1);
    matvec(&p2, y, M2);
    /* q = u - 1/2 and min(u, 1-u) from the integer stream value, in FP32 */
    const float normf = (float)(1.0 / 4294967088.0);
    for (int64_t i = 0; i < count; ++i) {
        const uint32_t zi = next_z(x, y);
        const float q = (float)(int32_t)((int64_t)zi - 2147483544) * normf;
        const uint32_t zt = zi < 4294967088u - zi ? zi : 4294967088u - zi;
        const float pt = (float)zt * normf;
        z[i] = mean + sd * lmmo_ppnd7(q, pt);
    }
}

void lmmo_ppnd16_array(const double *p, int64_t n, double *x)
{
    for (int64_t i = 0; i < n; ++i) x[i] = lmmo_ppnd16(p[i]);
}
