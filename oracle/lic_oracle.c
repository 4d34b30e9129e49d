/*
 * lic_oracle.c -- CPU restatement of rLIC's line integral convolution.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests, the smoke
 * check and the CPU-baseline leg of the benchmark call it to check or time the
 * CUDA path.  The product path never links, loads or calls it.
 *
 * It restates, in plain C11, the arithmetic of the reference's native core
 * (neutrinoceros/rlic v0.5.3, src/lib.rs), with every operation that the
 * reference rounds separately rounded separately here (build with
 * -ffp-contract=off) and every `mul_add` written as fma()/fmaf():
 *
 *   time_to_next_pixel      src/lib.rs:157-180   (4 variants: fma x branchless)
 *   update_state            src/lib.rs:209-233
 *   advance                 src/lib.rs:236-273
 *   BoundaryPair/Set apply  src/lib.rs:83-96, 112-116
 *   convole_single_pixel    src/lib.rs:305-362
 *   convolve                src/lib.rs:364-406
 *   convolve_iteratively    src/lib.rs:408-443
 *
 * Variant bits (`variant` argument): bit 0 = the `fma` Cargo feature, bit 1 =
 * the `branchless` feature (Cargo.toml:27-30).  The reference's default build
 * has both on (variant 3), which is the parity target.
 *
 * Indices follow the reference exactly: pixel coordinates are size_t and a
 * step left from 0 wraps to SIZE_MAX (Rust `usize::wrapping_sub`) before the
 * boundary rule maps it back into the image.
 *
 * Rows are independent within one iteration, so the OpenMP loop over rows
 * gives results bit-identical to the serial double loop of src/lib.rs:373-374.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_FMA 1u
#define ORACLE_BRANCHLESS 2u

/* boundary kinds: src/lib.rs:56-59 */
#define B_CLOSED 0
#define B_PERIODIC 1

/* apply_one_dir: src/lib.rs:83-96.  The fraction is deliberately untouched. */
static inline void apply_one_dir(size_t *c, int left, int right, size_t size) {
    if (*c == SIZE_MAX) {
        *c = (left == B_CLOSED) ? 0 : size - 1;
    } else if (*c == size) {
        *c = (right == B_CLOSED) ? size - 1 : 0;
    }
}

typedef struct {
    int xl, xr, yl, yr;
    size_t nx, ny; /* nx = number of columns (u.shape[1]), ny = rows */
} bounds_t;

/* BoundarySet::apply, src/lib.rs:112-116: x acts on j, y acts on i. */
static inline void apply_bounds(const bounds_t *b, size_t *i, size_t *j) {
    apply_one_dir(j, b->xl, b->xr, b->nx);
    apply_one_dir(i, b->yl, b->yr, b->ny);
}

/*
 * The same algorithm is instantiated for float and double by the macro below.
 * T = element type, S = suffix, FMA_ = fma function, FABS_ = fabs function.
 */
#define DEFINE_ORACLE(T, S, FMA_, FABS_)                                                 \
                                                                                         \
    /* num-traits Signed::signum for floats: NaN -> NaN, sign bit -> -1, else +1 */      \
    static inline T signum_##S(T x) {                                                    \
        if (isnan(x)) return x;                                                          \
        return signbit(x) ? (T)-1 : (T)1;                                                \
    }                                                                                    \
                                                                                         \
    /* time_to_next_pixel, src/lib.rs:157-180 */                                         \
    T lic_oracle_time_to_next_pixel_##S(T velocity, T frac, unsigned variant) {          \
        const T one = (T)1, half = (T)0.5;                                               \
        if (!(variant & ORACLE_BRANCHLESS)) {                                            \
            if (velocity > (T)0) return (one - frac) / velocity;                         \
            if (velocity < (T)0) return -(frac / velocity);                              \
            return (T)INFINITY;                                                          \
        }                                                                                \
        T s = one + signum_##S(velocity);                                                \
        T rem;                                                                           \
        if (variant & ORACLE_FMA)                                                        \
            rem = FMA_(s, half - frac, frac);                                            \
        else                                                                             \
            rem = s * (half - frac) + frac;                                              \
        return FABS_(rem / velocity);                                                    \
    }                                                                                    \
                                                                                         \
    /* update_state, src/lib.rs:209-233 */                                               \
    static inline void update_state_##S(T vpar, T vorth, size_t *cpar, T *fpar,          \
                                        T *forth, T tpar, unsigned variant) {            \
        if (vpar >= (T)0) {                                                              \
            *cpar += 1;                                                                  \
            *fpar = (T)0;                                                                \
        } else {                                                                         \
            *cpar -= 1; /* wraps to SIZE_MAX like usize::wrapping_sub */                 \
            *fpar = (T)1;                                                                \
        }                                                                                \
        if (variant & ORACLE_FMA)                                                        \
            *forth = FMA_(tpar, vorth, *forth);                                          \
        else                                                                             \
            *forth += tpar * vorth;                                                      \
    }                                                                                    \
                                                                                         \
    /* advance, src/lib.rs:236-273 */                                                    \
    void lic_oracle_advance_##S(T u, T v, size_t *i, size_t *j, T *fx, T *fy,            \
                                const bounds_t *b, unsigned variant) {                   \
        if (u == (T)0 && v == (T)0) return;                                              \
        T tx = lic_oracle_time_to_next_pixel_##S(u, *fx, variant);                       \
        T ty = lic_oracle_time_to_next_pixel_##S(v, *fy, variant);                       \
        if (tx < ty)                                                                     \
            update_state_##S(u, v, j, fx, fy, tx, variant);                              \
        else                                                                             \
            update_state_##S(v, u, i, fy, fx, ty, variant);                              \
        apply_bounds(b, i, j);                                                           \
    }                                                                                    \
                                                                                         \
    /* convole_single_pixel, src/lib.rs:305-362.  When path_i/path_j are given,  */      \
    /* the cell reached by every step is recorded; returns the number of steps.  */      \
    static int64_t trace_##S(T *acc, size_t i0, size_t j0, const T *u, const T *v,       \
                             const T *kernel, size_t klen, const T *input,               \
                             const bounds_t *b, int polarization, int backward,          \
                             unsigned variant, int64_t *path_i, int64_t *path_j) {       \
        size_t i = i0, j = j0;                                                           \
        T fx = (T)0.5, fy = (T)0.5;                                                      \
        T lu = (T)0, lv = (T)0;                                                          \
        const size_t nx = b->nx;                                                         \
        size_t kmid = klen / 2;                                                          \
        int64_t nsteps = 0;                                                              \
        size_t count = backward ? kmid : (klen > kmid + 1 ? klen - kmid - 1 : 0);        \
        for (size_t s = 0; s < count; ++s) {                                             \
            size_t k = backward ? kmid - 1 - s : kmid + 1 + s;                           \
            T pu = u[i * nx + j], pv = v[i * nx + j];                                    \
            if (isnan(pu) || isnan(pv)) break;                                           \
            if (polarization) {                                                          \
                T pu_lu = pu * lu;                                                       \
                T pv_lv = pv * lv;                                                       \
                if (pu_lu + pv_lv < (T)0) {                                              \
                    pu = -pu;                                                            \
                    pv = -pv;                                                            \
                }                                                                        \
                lu = pu;                                                                 \
                lv = pv;                                                                 \
            }                                                                            \
            if (backward) {                                                              \
                pu = -pu;                                                                \
                pv = -pv;                                                                \
            }                                                                            \
            lic_oracle_advance_##S(pu, pv, &i, &j, &fx, &fy, b, variant);                \
            T x = input[i * nx + j];                                                     \
            if (variant & ORACLE_FMA)                                                    \
                *acc = FMA_(kernel[k], x, *acc);                                         \
            else                                                                         \
                *acc += kernel[k] * x;                                                   \
            if (path_i) {                                                                \
                path_i[nsteps] = (int64_t)i;                                             \
                path_j[nsteps] = (int64_t)j;                                             \
            }                                                                            \
            ++nsteps;                                                                    \
        }                                                                                \
        return nsteps;                                                                   \
    }                                                                                    \
                                                                                         \
    /* convolve, src/lib.rs:364-406: one full sweep into a zeroed output */              \
    static void sweep_##S(const T *u, const T *v, const T *kernel, size_t klen,          \
                          const T *input, T *output, const bounds_t *b,                  \
                          int polarization, unsigned variant, int nthreads) {            \
        const size_t kmid = klen / 2;                                                    \
        const long long ny = (long long)b->ny;                                           \
        (void)nthreads;                                                                  \
        _Pragma("omp parallel for schedule(dynamic, 1) num_threads(nthreads)")          \
        for (long long ii = 0; ii < ny; ++ii) {                                          \
            size_t i = (size_t)ii;                                                       \
            for (size_t j = 0; j < b->nx; ++j) {                                         \
                T acc = output[i * b->nx + j];                                           \
                T x = input[i * b->nx + j];                                              \
                if (variant & ORACLE_FMA)                                                \
                    acc = FMA_(kernel[kmid], x, acc);                                    \
                else                                                                     \
                    acc += kernel[kmid] * x;                                             \
                trace_##S(&acc, i, j, u, v, kernel, klen, input, b, polarization, 0,     \
                          variant, NULL, NULL);                                          \
                trace_##S(&acc, i, j, u, v, kernel, klen, input, b, polarization, 1,     \
                          variant, NULL, NULL);                                          \
                output[i * b->nx + j] = acc;                                             \
            }                                                                            \
        }                                                                                \
    }                                                                                    \
                                                                                         \
    /* convolve_iteratively, src/lib.rs:408-443.  u, v, texture, out are C-order */      \
    /* (ny, nx).  iterations <= 0 leaves `out` zeroed, as the native core does.   */     \
    int lic_oracle_convolve_##S(const T *texture, const T *u, const T *v, int64_t ny,    \
                                int64_t nx, const T *kernel, int64_t klen,               \
                                int polarization, int xl, int xr, int yl, int yr,        \
                                int64_t iterations, T *out, unsigned variant,            \
                                int nthreads) {                                          \
        if (ny <= 0 || nx <= 0 || klen <= 0) return -1;                                  \
        size_t n = (size_t)ny * (size_t)nx;                                              \
        bounds_t b = {xl, xr, yl, yr, (size_t)nx, (size_t)ny};                           \
        T *input = (T *)malloc(n * sizeof(T));                                           \
        if (!input) return -2;                                                           \
        memcpy(input, texture, n * sizeof(T));                                           \
        memset(out, 0, n * sizeof(T));                                                   \
        if (nthreads <= 0) nthreads = 1;                                                 \
        for (int64_t it = 0; it < iterations; ++it) {                                    \
            sweep_##S(u, v, kernel, (size_t)klen, input, out, &b, polarization,          \
                      variant, nthreads);                                                \
            if (it + 1 < iterations) {                                                   \
                memcpy(input, out, n * sizeof(T));                                       \
                memset(out, 0, n * sizeof(T));                                           \
            }                                                                            \
        }                                                                                \
        free(input);                                                                     \
        return 0;                                                                        \
    }                                                                                    \
                                                                                         \
    /* One pass over the rows [row0, row1) only: the CPU baseline times a band  */      \
    /* of a large image with this.  `out` holds rows [row0, row1).              */      \
    int lic_oracle_sweep_rows_##S(const T *texture, const T *u, const T *v, int64_t ny,  \
                                  int64_t nx, const T *kernel, int64_t klen,             \
                                  int polarization, int xl, int xr, int yl, int yr,      \
                                  int64_t row0, int64_t row1, T *out, unsigned variant,  \
                                  int nthreads) {                                        \
        if (ny <= 0 || nx <= 0 || klen <= 0 || row0 < 0 || row1 > ny || row0 > row1)     \
            return -1;                                                                   \
        bounds_t b = {xl, xr, yl, yr, (size_t)nx, (size_t)ny};                           \
        const size_t kmid = (size_t)klen / 2;                                            \
        if (nthreads <= 0) nthreads = 1;                                                 \
        _Pragma("omp parallel for schedule(dynamic, 1) num_threads(nthreads)")          \
        for (long long ii = row0; ii < row1; ++ii) {                                     \
            size_t i = (size_t)ii;                                                       \
            for (size_t j = 0; j < (size_t)nx; ++j) {                                    \
                T acc = (T)0;                                                            \
                T x = texture[i * (size_t)nx + j];                                       \
                if (variant & ORACLE_FMA)                                                \
                    acc = FMA_(kernel[kmid], x, acc);                                    \
                else                                                                     \
                    acc += kernel[kmid] * x;                                             \
                trace_##S(&acc, i, j, u, v, kernel, (size_t)klen, texture, &b,           \
                          polarization, 0, variant, NULL, NULL);                         \
                trace_##S(&acc, i, j, u, v, kernel, (size_t)klen, texture, &b,           \
                          polarization, 1, variant, NULL, NULL);                         \
                out[(i - (size_t)row0) * (size_t)nx + j] = acc;                          \
            }                                                                            \
        }                                                                                \
        return 0;                                                                        \
    }                                                                                    \
                                                                                         \
    /* Cells visited by the streamlines of `npix` pixels.  For pixel p, slots   */      \
    /* [p*(klen-1), p*(klen-1)+nf) hold the forward trace (nf = klen-kmid-1)    */      \
    /* and the next kmid slots the backward trace; slots after a NaN stop hold  */      \
    /* -1.  Linear cell index i*nx+j.                                           */      \
    int lic_oracle_paths_##S(const T *u, const T *v, int64_t ny, int64_t nx,             \
                             int64_t klen, int polarization, int xl, int xr, int yl,     \
                             int yr, int64_t npix, const int64_t *pix, int64_t *cells,   \
                             unsigned variant) {                                         \
        if (ny <= 0 || nx <= 0 || klen <= 0) return -1;                                  \
        bounds_t b = {xl, xr, yl, yr, (size_t)nx, (size_t)ny};                           \
        size_t kmid = (size_t)klen / 2;                                                  \
        size_t nf = (size_t)klen - kmid - 1;                                             \
        size_t steps = (size_t)klen - 1;                                                 \
        int64_t *pi = (int64_t *)malloc((steps + 1) * sizeof(int64_t));                  \
        int64_t *pj = (int64_t *)malloc((steps + 1) * sizeof(int64_t));                  \
        T *zeros = (T *)calloc((size_t)klen, sizeof(T));                                 \
        if (!pi || !pj || !zeros) {                                                      \
            free(pi); free(pj); free(zeros);                                             \
            return -2;                                                                   \
        }                                                                                \
        for (int64_t p = 0; p < npix; ++p) {                                             \
            int64_t *dst = cells + p * (int64_t)steps;                                   \
            for (size_t s = 0; s < steps; ++s) dst[s] = -1;                              \
            size_t i = (size_t)(pix[p] / nx), j = (size_t)(pix[p] % nx);                 \
            T acc = (T)0;                                                                \
            /* the texture is irrelevant to the path: sample the zero kernel */          \
            int64_t n = trace_##S(&acc, i, j, u, v, zeros, (size_t)klen, u, &b,          \
                                  polarization, 0, variant, pi, pj);                     \
            for (int64_t s = 0; s < n; ++s) dst[s] = pi[s] * nx + pj[s];                 \
            n = trace_##S(&acc, i, j, u, v, zeros, (size_t)klen, u, &b, polarization,    \
                          1, variant, pi, pj);                                           \
            for (int64_t s = 0; s < n; ++s) dst[nf + (size_t)s] = pi[s] * nx + pj[s];    \
        }                                                                                \
        free(pi); free(pj); free(zeros);                                                 \
        return 0;                                                                        \
    }

DEFINE_ORACLE(float, f32, fmaf, fabsf)
DEFINE_ORACLE(double, f64, fma, fabs)

/* advance() on a single state, for the known-answer tests of src/lib.rs:275-297. */
int lic_oracle_advance_state_f64(double u, double v, int64_t *i, int64_t *j, double *fx,
                                 double *fy, int64_t ny, int64_t nx, int xl, int xr, int yl,
                                 int yr, unsigned variant) {
    bounds_t b = {xl, xr, yl, yr, (size_t)nx, (size_t)ny};
    size_t ii = (size_t)*i, jj = (size_t)*j;
    lic_oracle_advance_f64(u, v, &ii, &jj, fx, fy, &b, variant);
    *i = (int64_t)ii;
    *j = (int64_t)jj;
    return 0;
}

int lic_oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
