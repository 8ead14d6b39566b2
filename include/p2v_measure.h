/*
 * p2v_measure.h — measurement helpers of libp2v.so (not part of the drop-in boundary: no MegaMol module binds
 * them). They measure the hardware rates the benchmark's roofline figures divide by.
 */
#ifndef P2V_MEASURE_H
#define P2V_MEASURE_H

#include "p2v.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Texture sample rate of the current device for the learned AO's feature format (a layered texture of 8-bit
 * UNORM pairs, bilinear filtering, normalised coordinates), in G samples per second over a 128^3 level:
 *   pattern 0: the four lanes of every quad read adjacent texels of one layer (the units' coherent rate);
 *   pattern 1: every lane reads its own random point of a 64^3 region (different layers), the access pattern of
 *              cone samples whose directions follow each particle's normal.
 * Runs a few milliseconds of kernels on the calling thread's current device and stream 0. */
P2V_API p2v_status p2v_measure_texture_rate(int pattern, double* gsamples_per_s);

#ifdef __cplusplus
}
#endif

#endif
