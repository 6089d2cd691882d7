/*
 * lombscargle_py.h -- the reference-compatible C ABI.
 *
 * Exported, with this exact signature, by each of the four drop-in libraries
 *   libpylsnoerrorfloat.so   (ERROR=0, DTYPE=float)
 *   libpylsnoerrordouble.so  (ERROR=0, DTYPE=double)
 *   libpylserrorfloat.so     (ERROR=1, DTYPE=float)
 *   libpylserrordouble.so    (ERROR=1, DTYPE=double)
 * It replaces source/main.cu:255-411 (LombScarglePy, built by source/Makefile:71-91
 * with -DPYTHON -DNORMALIZEPGRAM=1 -DRETURNPGRAM=1) and is bound by
 * source/lombscarglegpu.py:337-364 through numpy.ctypeslib.
 *
 * Arguments (all caller-owned, C-contiguous):
 *   objectId[sizeData]  object ids; an object is a run of equal ids.
 *   timeX, magY, magDY  [sizeData] DTYPE; magDY is read only when ERROR=1.
 *   minFreq, maxFreq    angular frequencies (rad/time), maxFreq exclusive.
 *   freqToTest          number of frequencies N.
 *   MODE                1 GPU batch, 2 GPU single object (all rows), 4 CPU batch,
 *                       5 CPU single object; any other value computes nothing.
 *   pgram               [num_objects x N] DTYPE output, written in full:
 *                       ERROR=0 normalized by 2/(N_obs var(y)); ERROR=1 as computed.
 * Side effects kept from the reference: with ERROR=1 magY is pre-centered in place
 * (y -= sum(y/sqrt(dy))/sum(1/sqrt(dy)), per object; source/main.cu:1631-1662);
 * progress lines go to stdout; a line is appended to gpu_stats.txt in the working
 * directory unless LSGB_NO_STATS=1.
 * Errors: the reference exits the process on a CUDA error (source/main.cu:38-46).
 * Here a failure prints "GPUassert"-style text to stderr, leaves pgram as it was and
 * returns; LombScarglePy_last_status() then returns the negative lsgb status.
 * Setting LSGB_EXIT_ON_ERROR=1 restores the reference's exit(code).
 */
#ifndef LOMBSCARGLE_PY_H
#define LOMBSCARGLE_PY_H

#ifdef __cplusplus
extern "C" {
#endif

#ifndef LS_DTYPE
#define LS_DTYPE double
#endif

__attribute__((visibility("default"))) void LombScarglePy(unsigned int *objectId, LS_DTYPE *timeX,
                                                          LS_DTYPE *magY, LS_DTYPE *magDY,
                                                          unsigned int sizeData, double minFreq,
                                                          double maxFreq, unsigned int freqToTest,
                                                          int MODE, LS_DTYPE *pgram);

/* Status of the last LombScarglePy call on this thread (0 ok, lsgb status otherwise).
 * No counterpart in the reference, whose entry point has no error reporting. */
__attribute__((visibility("default"))) int LombScarglePy_last_status(void);

#ifdef __cplusplus
}
#endif

#endif
