// lsgb_cpu.h -- the reference ABI's CPU modes (MODE 4: batch, MODE 5: one object).
//
// These modes are part of LombScarglePy's contract (source/main.cu:360-394): a
// caller asks for them explicitly and they never run in place of a GPU mode. The
// arithmetic follows the reference's CPU path in the library's DTYPE, including
// its mixed float/double promotions, so the float builds reproduce the float
// reference:
//   standard    source/main.cu:1566-1599 (lombscarglecpuinnerloop)
//   generalized source/main.cu:1701-1777 (lombscarglecpuinnerloopAstroPy)
//   pre-center  source/main.cu:1631-1662 (updateYerrorfactor, w = 1/sqrt(dy))
//   normalize   source/main.cu:1295-1352;  argmax/period source/main.cu:1545-1563
// OpenMP parallelism: objects (MODE 4, dynamic schedule) or frequencies (MODE 5),
// as in source/main.cu:1487 and :1617.
#pragma once

#include <stdint.h>

#include <cmath>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace lsgb_cpu {

template <typename T>
T power_std(const T *x, const T *y, uint32_t n, T w) {
    T c, s, xc = 0.0, xs = 0.0, cc = 0.0, ss = 0.0, cs = 0.0;
    for (uint32_t j = 0; j < n; j++) {
        c = std::cos(w * x[j]);
        s = std::sin(w * x[j]);
        xc += y[j] * c;
        xs += y[j] * s;
        cc += c * c;
        ss += s * s;
        cs += c * s;
    }
    T tau = std::atan2(2.0 * cs, cc - ss) / (2.0 * w);
    T c_tau = std::cos(w * tau);
    T s_tau = std::sin(w * tau);
    T c_tau2 = c_tau * c_tau;
    T s_tau2 = s_tau * s_tau;
    T cs_tau = 2.0 * c_tau * s_tau;
    return 0.5 * ((((c_tau * xc + s_tau * xs) * (c_tau * xc + s_tau * xs)) /
                   (c_tau2 * cc + cs_tau * cs + s_tau2 * ss)) +
                  (((c_tau * xs - s_tau * xc) * (c_tau * xs - s_tau * xc)) /
                   (c_tau2 * ss - cs_tau * cs + s_tau2 * cc)));
}

template <typename T>
T power_gen(const T *x, const T *y, const T *dy, uint32_t n, T f) {
    T w, omega_t, sin_omega_t, cos_omega_t, S = 0.0, C = 0.0, S2 = 0.0, C2 = 0.0, wsum = 0.0;
    for (uint32_t j = 0; j < n; j++) {
        w = 1.0 / dy[j];
        w *= w;
        wsum += w;
        omega_t = f * x[j];
        sin_omega_t = std::sin(omega_t);
        cos_omega_t = std::cos(omega_t);
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
    T tau = 0.5 * std::atan2(S2, C2) / f;
    T Y = 0.0, YY = 0.0, Stau = 0.0, Ctau = 0.0, YCtau = 0.0, YStau = 0.0, CCtau = 0.0, SStau = 0.0;
    for (uint32_t j = 0; j < n; j++) {
        w = 1.0 / dy[j];
        w *= w;
        omega_t = f * (x[j] - tau);
        sin_omega_t = std::sin(omega_t);
        cos_omega_t = std::cos(omega_t);
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

// y -= sum(w*y)/sum(w), w = 1/sqrt(dy), in place; sums kept in DTYPE as the
// reference does (its OpenMP reduction order is not reproduced).
template <typename T>
void precenter(T *y, const T *dy, uint32_t n) {
    T sumw = 0, dotwy = 0;
    for (uint32_t i = 0; i < n; i++) {
        T w = 1.0 / std::sqrt(dy[i]);
        sumw += w;
        dotwy += w * y[i];
    }
    for (uint32_t i = 0; i < n; i++) y[i] = y[i] - dotwy / sumw;
}

template <typename T>
double var_pop(const T *y, uint64_t n) {
    double sum = 0;
    for (uint64_t k = 0; k < n; k++) sum += y[k];
    double mean = sum / (n * 1.0);
    double sum2 = 0;
    for (uint64_t k = 0; k < n; k++) sum2 += (y[k] - mean) * (y[k] - mean);
    double sigma = std::sqrt(sum2 / (n * 1.0));
    return sigma * sigma;
}

template <typename T>
void argmax(const T *p, uint32_t nf, T minFreq, T freqStep, T *period, T *power) {
    T maxPower = 0;
    uint32_t maxIdx = 0;
    for (uint32_t i = 0; i < nf; i++)
        if (maxPower < p[i]) {
            maxPower = p[i];
            maxIdx = i;
        }
    *period = (1.0 / (minFreq + (maxIdx * freqStep))) * 2.0 * M_PI;
    *power = maxPower;
}

// One object's full periodogram into pg[0..nf), normalized for the standard variant.
template <typename T, int ERR>
void object_pgram(const T *x, T *y, const T *dy, uint32_t n, uint32_t nf, T minFreq, T freqStep,
                  T *pg, bool parallel_freqs) {
    if (ERR) precenter(y, dy, n);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (parallel_freqs)
#endif
    for (uint32_t i = 0; i < nf; i++) {
        T f = minFreq + (freqStep * i);
        pg[i] = ERR ? power_gen<T>(x, y, dy, n, f) : power_std<T>(x, y, n, f);
    }
    if (!ERR) {
        const double scale = 2.0 / (n * var_pop(y, n));
        for (uint32_t j = 0; j < nf; j++) pg[j] *= scale;
    }
}

// MODE 4: objects are runs of equal id; returns the sum of the best periods.
template <typename T, int ERR>
double batch(const uint32_t *ids, const T *x, T *y, const T *dy, uint32_t rows, T minFreq, T maxFreq,
             uint32_t nf, T *pgram, uint32_t *n_obj_out) {
    std::vector<uint32_t> start{0};
    for (uint32_t i = 1; i < rows; i++)
        if (ids[i] != ids[i - 1]) start.push_back(i);
    start.push_back(rows);
    const uint32_t nobj = (uint32_t)start.size() - 1;
    *n_obj_out = nobj;
    const T freqStep = (maxFreq - minFreq) / (nf * 1.0);
    std::vector<T> period(nobj), power(nobj);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic)
#endif
    for (uint32_t o = 0; o < nobj; o++) {
        const uint32_t a = start[o], n = start[o + 1] - start[o];
        T *pg = pgram + (uint64_t)o * nf;
        object_pgram<T, ERR>(x + a, y + a, dy + a, n, nf, minFreq, freqStep, pg, false);
        argmax(pg, nf, minFreq, freqStep, &period[o], &power[o]);
    }
    double sum = 0;
    for (uint32_t o = 0; o < nobj; o++) sum += period[o];
    return sum;
}

// MODE 5: all rows are one object.
template <typename T, int ERR>
void single(const T *x, T *y, const T *dy, uint32_t rows, T minFreq, T maxFreq, uint32_t nf,
            T *pgram, T *period, T *power) {
    const T freqStep = (maxFreq - minFreq) / (nf * 1.0);
    object_pgram<T, ERR>(x, y, dy, rows, nf, minFreq, freqStep, pgram, true);
    argmax(pgram, nf, minFreq, freqStep, period, power);
}

}  // namespace lsgb_cpu
