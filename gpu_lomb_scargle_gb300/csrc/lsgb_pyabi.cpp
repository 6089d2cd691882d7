// lsgb_pyabi.cpp -- LombScarglePy, the reference's C ABI (source/main.cu:255-411).
//
// Compiled four times, -DLS_ERROR={0,1} -DLS_DTYPE={float,double}, into
// libpyls{noerror,error}{float,double}.so, which source/lombscarglegpu.py loads
// through ctypes unchanged. MODE 1 / 2 run on the GPU engine (lsgb_engine.cpp);
// MODE 4 / 5 are the reference's CPU modes (lsgb_cpu.h).
//
// Precision of the GPU modes: the double builds use the plain FP64 form (the
// reference double build's arithmetic, FP64 atan2 included); the float builds use
// the mixed form (FP64 phase anchors, FP32 recurrence), which is far closer to the
// FP64 result than the reference's float build (fast-math sincosf on phases up to
// 1e5-1e8 rad). LSGB_PRECISION=plain|mixed overrides the choice.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <cmath>
#include <fstream>
#include <mutex>
#include <vector>

#include "../../include/lsgb.h"
#include "../../include/lombscargle_py.h"
#include "lsgb_cpu.h"

#ifndef LS_ERROR
#error "LS_ERROR must be defined (0 or 1)"
#endif

typedef LS_DTYPE DTYPE;
#define LS_STR2(x) #x
#define LS_STR(x) LS_STR2(x)

namespace {

constexpr bool kIsFloat = sizeof(DTYPE) == 4;
thread_local int g_status = 0;
std::mutex g_eng_mu;
lsgb_engine *g_eng = nullptr;  // created by the first GPU call, lives until process exit

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int precision_choice() {
    const char *p = getenv("LSGB_PRECISION");
    if (p && !strcmp(p, "plain")) return LSGB_PLAIN_FP64;
    if (p && !strcmp(p, "mixed")) return LSGB_MIXED;
    return kIsFloat ? LSGB_MIXED : LSGB_PLAIN_FP64;
}

void report_failure(int rc) {
    g_status = rc;
    fprintf(stderr, "GPUassert: %s %s %d\n", lsgb_last_error(), __FILE__, __LINE__);
    const char *ex = getenv("LSGB_EXIT_ON_ERROR");
    if (ex && !strcmp(ex, "1")) exit(rc < 0 ? -rc : rc);
}

void append_stats(double secs, double val, double minFreq, double maxFreq, unsigned nf, int mode) {
    const char *no = getenv("LSGB_NO_STATS");
    if (no && !strcmp(no, "1")) return;
    std::ofstream f("gpu_stats.txt", std::ios::app);
    f << secs << ", Sum of periods: " << val << ", Min/Max Freq: " << minFreq << "/" << maxFreq
      << ",  Num tested freq: " << nf << ", MODE: " << mode << ", ERROR/DTYPE/ENGINE: " << LS_ERROR
      << ", " << LS_STR(LS_DTYPE) << ", lsgb" << std::endl;
}

}  // namespace

extern "C" int LombScarglePy_last_status(void) { return g_status; }

extern "C" void LombScarglePy(unsigned int *objectId, DTYPE *timeX, DTYPE *magY, DTYPE *magDY,
                              unsigned int sizeData, double minFreq, double maxFreq,
                              unsigned int freqToTest, int MODE, DTYPE *pgram) {
    g_status = 0;
    printf("\nMinimum Frequency: %f", minFreq);
    printf("\nMaximum Frequency: %f", maxFreq);
    printf("\nNumber of frequencies to test: %u", freqToTest);
    printf("\nMode: %d", MODE);
    if (LS_ERROR) printf("\nExecuting L-S variant from AstroPy that propogates error and floats the mean");
    if (MODE != 1 && MODE != 2 && MODE != 4 && MODE != 5) {
        fflush(stdout);
        return;
    }
    if (sizeData == 0 || !timeX || !magY || !pgram || (MODE != 2 && MODE != 5 && !objectId) ||
        (LS_ERROR && !magDY)) {
        g_status = LSGB_ERR_INVALID;
        fprintf(stderr, "LombScarglePy: empty input or NULL array\n");
        return;
    }
    // The reference's drivers take the limits as DTYPE (source/main.cu:742, :1358).
    const DTYPE fminT = (DTYPE)minFreq, fmaxT = (DTYPE)maxFreq;
    const double t0 = now_s();

    if (MODE == 4 || MODE == 5) {
        double val = 0;
        if (MODE == 4) {
            uint32_t nobj = 0;
            val = lsgb_cpu::batch<DTYPE, LS_ERROR>(objectId, timeX, magY, magDY, sizeData, fminT,
                                                   fmaxT, freqToTest, pgram, &nobj);
            printf("\nTotal time to compute batch: %f", now_s() - t0);
            printf("\n[Validation] Sum of all periods: %f", val);
        } else {
            DTYPE period = 0, power = 0;
            lsgb_cpu::single<DTYPE, LS_ERROR>(timeX, magY, magDY, sizeData, fminT, fmaxT, freqToTest,
                                              pgram, &period, &power);
            val = period;
            printf("\nTotal time to compute pgram (one object): %f", now_s() - t0);
            printf("\n[Validation] Period: %f, Power: %f", (double)period, (double)power);
        }
        fflush(stdout);
        append_stats(now_s() - t0, val, minFreq, maxFreq, freqToTest, MODE);
        return;
    }

    // ---- GPU modes ----
    std::vector<uint64_t> offsets{0};
    if (MODE == 1) {
        for (uint32_t i = 1; i < sizeData; i++)
            if (objectId[i] != objectId[i - 1]) offsets.push_back(i);
    }
    offsets.push_back(sizeData);
    const uint32_t nobj = (uint32_t)offsets.size() - 1;
    printf("\nNumber of unique objects: %u", nobj);
    if (LS_ERROR) {
        for (uint32_t o = 0; o < nobj; o++)
            lsgb_cpu::precenter<DTYPE>(magY + offsets[o], magDY + offsets[o],
                                       (uint32_t)(offsets[o + 1] - offsets[o]));
    }
    // Grid as the reference's kernels evaluate it: minFreq + freqStep*k with freqStep
    // = (maxFreq - minFreq)/N computed in double and held in DTYPE (source/kernel.cu:517).
    const double fmin = (double)fminT;
    const double df = (double)(DTYPE)(((double)fmaxT - (double)fminT) / (freqToTest * 1.0));

    int rc;
    {
        std::lock_guard<std::mutex> lk(g_eng_mu);
        if (!g_eng) {
            rc = lsgb_engine_create(0, &g_eng);
            if (rc != LSGB_OK) {
                report_failure(rc);
                return;
            }
        }
        std::vector<uint32_t> best(nobj);
        const int dtype = kIsFloat ? LSGB_F32 : LSGB_F64;
        const double tk = now_s();
        rc = lsgb_periodogram_host(g_eng, LS_ERROR ? LSGB_GENERALIZED : LSGB_STANDARD,
                                   precision_choice(), dtype, timeX, magY, LS_ERROR ? magDY : nullptr,
                                   offsets.data(), nobj, fmin, df, freqToTest, LS_ERROR ? 0 : 1,
                                   pgram, best.data(), nullptr);
        if (rc != LSGB_OK) {
            report_failure(rc);
            return;
        }
        printf("\nTime to compute kernel: %f", now_s() - tk);
        double val = 0;
        for (uint32_t o = 0; o < nobj; o++) val += (1.0 / (fmin + (best[o] * df))) * 2.0 * M_PI;
        if (MODE == 1) {
            printf("\nTotal time to compute batch: %f", now_s() - t0);
            printf("\n[Validation] Sum of all periods: %f", val);
        } else {
            printf("\nTotal time to compute batch: %f", now_s() - t0);
            printf("\n[Validation] Period: %f, Power: %f", val, (double)pgram[best[0]]);
        }
        fflush(stdout);
        append_stats(now_s() - t0, val, minFreq, maxFreq, freqToTest, MODE);
    }
}
