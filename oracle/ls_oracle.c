/*
 * ls_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, FP64 restatement of the reference's CPU Lomb-Scargle path
 * (mgowanlock/gpu_lomb_scargle, source/main.cu, modes 4 and 5). It is the
 * checker for the CUDA engine: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load it. Nothing in the product
 * libraries links it or calls it.
 *
 * Each function names the reference lines it follows. The arithmetic keeps the
 * reference's order of operations so that, compiled without FMA contraction
 * (-ffp-contract=off), it reproduces the reference's double build to rounding
 * (checked against the reference's own CPU build, see tests/golden/).
 *
 * Differences from the reference, all deliberate:
 *  - frequencies can be evaluated on an explicit subset of grid indices, so
 *    large grids can be spot-checked (the grid formula is unchanged);
 *  - the pre-centering sums are sequential (the reference uses OpenMP
 *    reductions whose order depends on the thread count);
 *  - nothing is printed, no gpu_stats.txt is written, nothing leaks.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define LSO_API __attribute__((visibility("default")))

/* Frequency grid, source/main.cu:1364 and :1609-1611:
 *   freqStep = (maxFreq - minFreq) / numFreqs;  omega_k = minFreq + freqStep * k
 * Returned as the exact double the reference's double build evaluates. */
LSO_API double lso_omega(double fmin, double df, uint32_t k) { return fmin + (df * (double)k); }

/* Contiguous-run segmentation, source/main.cu:468-510. Returns the number of
 * objects; writes inclusive [idx_min, idx_max] ranges (up to cap entries). */
LSO_API uint32_t lso_object_ranges(const uint32_t *obj_id, uint32_t n, uint32_t *idx_min,
                                   uint32_t *idx_max, uint32_t cap) {
    if (n == 0) return 0;
    uint32_t cnt = 0;
    uint32_t last = obj_id[0];
    if (cap > 0) idx_min[0] = 0;
    for (uint32_t i = 1; i < n; i++) {
        if (obj_id[i] != last) {
            if (cnt < cap) idx_max[cnt] = i - 1;
            if (cnt + 1 < cap) idx_min[cnt + 1] = i;
            cnt++;
            last = obj_id[i];
        }
    }
    if (cnt < cap) idx_max[cnt] = n - 1;
    return cnt + 1;
}

/* Standard L-S power at one angular frequency, source/main.cu:1566-1599
 * (lombscarglecpuinnerloop), same statement order. */
LSO_API double lso_std_power(const double *x, const double *y, uint32_t n, double w) {
    double c, s, xc = 0.0, xs = 0.0, cc = 0.0, ss = 0.0, cs = 0.0;
    for (uint32_t j = 0; j < n; j++) {
        c = cos(w * x[j]);
        s = sin(w * x[j]);
        xc += y[j] * c;
        xs += y[j] * s;
        cc += c * c;
        ss += s * s;
        cs += c * s;
    }
    double tau = atan2(2.0 * cs, cc - ss) / (2.0 * w);
    double c_tau = cos(w * tau);
    double s_tau = sin(w * tau);
    double c_tau2 = c_tau * c_tau;
    double s_tau2 = s_tau * s_tau;
    double cs_tau = 2.0 * c_tau * s_tau;
    return 0.5 * ((((c_tau * xc + s_tau * xs) * (c_tau * xc + s_tau * xs)) /
                   (c_tau2 * cc + cs_tau * cs + s_tau2 * ss)) +
                  (((c_tau * xs - s_tau * xc) * (c_tau * xs - s_tau * xc)) /
                   (c_tau2 * ss - cs_tau * cs + s_tau2 * cc)));
}

/* Generalized (floating-mean, weighted) power, source/main.cu:1701-1777
 * (lombscarglecpuinnerloopAstroPy): a tau pass, then a power pass at
 * omega*(t - tau). Same statement order. */
LSO_API double lso_gen_power(const double *x, const double *y, const double *dy, uint32_t n,
                             double f) {
    double w, omega_t, sin_omega_t, cos_omega_t;
    double S = 0.0, C = 0.0, S2 = 0.0, C2 = 0.0, wsum = 0.0;
    for (uint32_t j = 0; j < n; j++) {
        w = 1.0 / dy[j];
        w *= w;
        wsum += w;
        omega_t = f * x[j];
        sin_omega_t = sin(omega_t);
        cos_omega_t = cos(omega_t);
        S += w * sin_omega_t;
        C += w * cos_omega_t;
        S2 += 2.0 * w * sin_omega_t * cos_omega_t;
        C2 += w - 2.0 * w * sin_omega_t * sin_omega_t;
    }
    S2 /= wsum;
    C2 /= wsum;
    S /= wsum;
    C /= wsum;
    S2 -= (2.0 * S * C);
    C2 -= (C * C - S * S);
    double tau = 0.5 * atan2(S2, C2) / f;
    double Y = 0.0, YY = 0.0, Stau = 0.0, Ctau = 0.0, YCtau = 0.0, YStau = 0.0, CCtau = 0.0,
           SStau = 0.0;
    for (uint32_t j = 0; j < n; j++) {
        w = 1.0 / dy[j];
        w *= w;
        omega_t = f * (x[j] - tau);
        sin_omega_t = sin(omega_t);
        cos_omega_t = cos(omega_t);
        Y += w * y[j];
        YY += w * y[j] * y[j];
        Ctau += w * cos_omega_t;
        Stau += w * sin_omega_t;
        YCtau += w * y[j] * cos_omega_t;
        YStau += w * y[j] * sin_omega_t;
        CCtau += w * cos_omega_t * cos_omega_t;
        SStau += w * sin_omega_t * sin_omega_t;
    }
    Y /= wsum;
    YY /= wsum;
    Ctau /= wsum;
    Stau /= wsum;
    YCtau /= wsum;
    YStau /= wsum;
    CCtau /= wsum;
    SStau /= wsum;
    YCtau -= Y * Ctau;
    YStau -= Y * Stau;
    CCtau -= Ctau * Ctau;
    SStau -= Stau * Stau;
    YY -= Y * Y;
    return (YCtau * YCtau / CCtau + YStau * YStau / SStau) / YY;
}

/* Pre-centering of y for the generalized variant, source/main.cu:1631-1662
 * (updateYerrorfactor). The reference's weights are 1/sqrt(dy) although its
 * comment says dy**-2; the oracle keeps the code's behaviour. In place. */
LSO_API void lso_precenter(double *y, const double *dy, uint32_t n) {
    double sumw = 0.0, dotwy = 0.0;
    for (uint32_t i = 0; i < n; i++) sumw += 1.0 / sqrt(dy[i]);
    for (uint32_t i = 0; i < n; i++) dotwy += (1.0 / sqrt(dy[i])) * y[i];
    for (uint32_t i = 0; i < n; i++) y[i] = y[i] - dotwy / sumw;
}

/* Normalization factor 2/(N*sigma^2) with the population variance of y,
 * source/main.cu:1295-1317 (computeStandardDevSquared) and :1335/:1350. */
LSO_API double lso_norm_factor(const double *y, uint32_t n) {
    double sum = 0.0;
    for (uint32_t k = 0; k < n; k++) sum += y[k];
    double mean = sum / (n * 1.0);
    double sum2 = 0.0;
    for (uint32_t k = 0; k < n; k++) sum2 += (y[k] - mean) * (y[k] - mean);
    double sigma = sqrt(sum2 / (n * 1.0));
    return 2.0 / (n * (sigma * sigma));
}

/* Best frequency, source/main.cu:1545-1563 (computePeriod): starts at power 0,
 * strict '<', so the first maximum wins and NaN / non-positive powers never do. */
LSO_API void lso_argmax(const double *p, uint32_t nf, uint32_t *idx, double *power) {
    double maxp = 0.0;
    uint32_t maxi = 0;
    for (uint32_t i = 0; i < nf; i++) {
        if (maxp < p[i]) {
            maxp = p[i];
            maxi = i;
        }
    }
    *idx = maxi;
    *power = maxp;
}

/* The three best frequencies, source/main.cu:1165-1219 (PRINTPERIODS==3): three
 * scans from (power 0, index 0), each with the strict '<' of the argmax, the second
 * skipping the first's index and the third skipping both earlier indices. */
LSO_API void lso_top3(const double *p, uint32_t nf, uint32_t *idx, double *power) {
    double maxp[3] = {0.0, 0.0, 0.0};
    uint32_t maxi[3] = {0, 0, 0};
    for (int r = 0; r < 3; r++) {
        for (uint32_t j = 0; j < nf; j++) {
            if (r >= 1 && j == maxi[0]) continue;
            if (r >= 2 && j == maxi[1]) continue;
            if (maxp[r] < p[j]) {
                maxp[r] = p[j];
                maxi[r] = j;
            }
        }
        idx[r] = maxi[r];
        power[r] = maxp[r];
    }
}

/* Batch periodogram on a subset of grid indices.
 *   variant 0: standard (source/main.cu:1469-1502, normalized when normalize!=0
 *              as the Python builds do, :1497-1499);
 *   variant 1: generalized, y pre-centered per object first (:1667-1672), the
 *              pre-centered y written back into y (the reference mutates the
 *              caller's array the same way).
 * Objects are the inclusive row ranges [idx_min[o], idx_max[o]]. out is
 * nobj x nk row-major. kidx==NULL means k = 0..nk-1. nthreads<=0: OpenMP default. */
LSO_API int lso_batch_pgram(int variant, const double *t, double *y, const double *dy,
                            const uint32_t *idx_min, const uint32_t *idx_max, uint32_t nobj,
                            double fmin, double df, const uint32_t *kidx, uint32_t nk,
                            int normalize, double *out, int nthreads) {
    if (variant != 0 && variant != 1) return -1;
    double *norm = (double *)malloc(sizeof(double) * (nobj ? nobj : 1));
    if (!norm) return -2;
    for (uint32_t o = 0; o < nobj; o++) {
        uint32_t a = idx_min[o], n = idx_max[o] - idx_min[o] + 1;
        if (variant == 1) lso_precenter(y + a, dy + a, n);
        norm[o] = (variant == 0 && normalize) ? lso_norm_factor(y + a, n) : 1.0;
    }
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for num_threads(nt) schedule(dynamic, 64) collapse(2)
#endif
    for (uint32_t o = 0; o < nobj; o++) {
        for (uint32_t q = 0; q < nk; q++) {
            uint32_t a = idx_min[o], n = idx_max[o] - idx_min[o] + 1;
            uint32_t k = kidx ? kidx[q] : q;
            double w = lso_omega(fmin, df, k);
            double p = variant == 0 ? lso_std_power(t + a, y + a, n, w)
                                    : lso_gen_power(t + a, y + a, dy + a, n, w);
            out[(uint64_t)o * nk + q] = p * norm[o];
        }
    }
    (void)nthreads;
    free(norm);
    return 0;
}

/* Number of OpenMP threads the oracle would use (for reporting core counts). */
LSO_API int lso_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
