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

// Standard power at angular frequency om. The statement order (and so the rounding, in
// float and double) is that of the reference's CPU loop: the five sums over the
// observations, the time shift that decouples the cosine and sine terms, then the two
// quotients of the tau-rotated form.
template <typename T>
T power_std(const T *x, const T *y, uint32_t n, T om) {
    T cw, sw, syc = 0.0, sys = 0.0, scc = 0.0, sss = 0.0, scs = 0.0;
    for (uint32_t j = 0; j < n; j++) {
        cw = std::cos(om * x[j]);
        sw = std::sin(om * x[j]);
        syc += y[j] * cw;
        sys += y[j] * sw;
        scc += cw * cw;
        sss += sw * sw;
        scs += cw * sw;
    }
    const T shift = std::atan2(2.0 * scs, scc - sss) / (2.0 * om);
    const T cr = std::cos(om * shift);
    const T sr = std::sin(om * shift);
    const T cr2 = cr * cr;
    const T sr2 = sr * sr;
    const T csr = 2.0 * cr * sr;
    const T along = cr * syc + sr * sys;    // projection on the shifted cosine
    const T across = cr * sys - sr * syc;   // and on the shifted sine
    const T quo_c = (along * along) / (cr2 * scc + csr * scs + sr2 * sss);
    const T quo_s = (across * across) / (cr2 * sss - csr * scs + sr2 * scc);
    return 0.5 * (quo_c + quo_s);
}

// Generalized power (floating mean, weights 1/dy^2) at angular frequency om: a first pass
// for the time shift from the weighted doubled-angle sums, a second at om (t - shift) for the
// weighted, mean-subtracted sums. Statement order as in the reference's CPU loop.
template <typename T>
T power_gen(const T *x, const T *y, const T *dy, uint32_t n, T om) {
    T wt, ph, sph, cph, m_s = 0.0, m_c = 0.0, m_s2 = 0.0, m_c2 = 0.0, wsum = 0.0;
    for (uint32_t j = 0; j < n; j++) {
        wt = 1.0 / dy[j];
        wt *= wt;
        wsum += wt;
        ph = om * x[j];
        sph = std::sin(ph);
        cph = std::cos(ph);
        m_s += wt * sph;
        m_c += wt * cph;
        m_s2 += 2.0 * wt * sph * cph;
        m_c2 += wt - 2.0 * wt * sph * sph;
    }
    m_s2 /= wsum;
    m_c2 /= wsum;
    m_s /= wsum;
    m_c /= wsum;
    m_s2 -= (2.0 * m_s * m_c);
    m_c2 -= (m_c * m_c - m_s * m_s);
    const T shift = 0.5 * std::atan2(m_s2, m_c2) / om;
    T my = 0.0, myy = 0.0, ms = 0.0, mc = 0.0, myc = 0.0, mys = 0.0, mcc = 0.0, mss = 0.0;
    for (uint32_t j = 0; j < n; j++) {
        wt = 1.0 / dy[j];
        wt *= wt;
        ph = om * (x[j] - shift);
        sph = std::sin(ph);
        cph = std::cos(ph);
        my += wt * y[j];
        myy += wt * y[j] * y[j];
        mc += wt * cph;
        ms += wt * sph;
        myc += wt * y[j] * cph;
        mys += wt * y[j] * sph;
        mcc += wt * cph * cph;
        mss += wt * sph * sph;
    }
    my /= wsum;
    myy /= wsum;
    mc /= wsum;
    ms /= wsum;
    myc /= wsum;
    mys /= wsum;
    mcc /= wsum;
    mss /= wsum;
    // covariances about the weighted means
    myc -= my * mc;
    mys -= my * ms;
    mcc -= mc * mc;
    mss -= ms * ms;
    myy -= my * my;
    return (myc * myc / mcc + mys * mys / mss) / myy;
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

// One object's full periodogram into pg[0..nf); the standard variant is normalized by
// 2/(N var(y)) when `normalize` (the Python builds, -DNORMALIZEPGRAM=1; the command line
// leaves it unnormalized unless asked, source/params.h:40).
template <typename T, int ERR>
void object_pgram(const T *x, T *y, const T *dy, uint32_t n, uint32_t nf, T minFreq, T freqStep,
                  T *pg, bool parallel_freqs, bool normalize = true) {
    if (ERR) precenter(y, dy, n);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) if (parallel_freqs)
#endif
    for (uint32_t i = 0; i < nf; i++) {
        T f = minFreq + (freqStep * i);
        pg[i] = ERR ? power_gen<T>(x, y, dy, n, f) : power_std<T>(x, y, n, f);
    }
    if (!ERR && normalize) {
        const double scale = 2.0 / (n * var_pop(y, n));
        for (uint32_t j = 0; j < nf; j++) pg[j] *= scale;
    }
}

// MODE 4: objects are runs of equal id; returns the sum of the best periods.
template <typename T, int ERR>
double batch(const uint32_t *ids, const T *x, T *y, const T *dy, uint32_t rows, T minFreq, T maxFreq,
             uint32_t nf, T *pgram, uint32_t *n_obj_out, bool normalize = true) {
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
        object_pgram<T, ERR>(x + a, y + a, dy + a, n, nf, minFreq, freqStep, pg, false, normalize);
        argmax(pg, nf, minFreq, freqStep, &period[o], &power[o]);
    }
    double sum = 0;
    for (uint32_t o = 0; o < nobj; o++) sum += period[o];
    return sum;
}

// MODE 5: all rows are one object.
template <typename T, int ERR>
void single(const T *x, T *y, const T *dy, uint32_t rows, T minFreq, T maxFreq, uint32_t nf,
            T *pgram, T *period, T *power, bool normalize = true) {
    const T freqStep = (maxFreq - minFreq) / (nf * 1.0);
    object_pgram<T, ERR>(x, y, dy, rows, nf, minFreq, freqStep, pgram, true, normalize);
    argmax(pgram, nf, minFreq, freqStep, period, power);
}

}  // namespace lsgb_cpu
