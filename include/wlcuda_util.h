/* wlcuda utilities: seeded synthetic inputs for the benchmark configurations. No counterpart in
 * the reference (its cases build their inputs from an integer hash, as these do); nothing on the
 * tick's path calls them. */
#ifndef WLCUDA_UTIL_H
#define WLCUDA_UTIL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* nx * ny heights in [0, height]: six-octave value-noise fBm on the reference's integer-hash
 * lattice (lacunarity 2, gain 0.5, base period max(nx, ny) / 4), normalised; 0 on success. */
int wl_util_fbm(double* out, uint32_t nx, uint32_t ny, double height, uint64_t seed,
                uint32_t octaves);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* WLCUDA_UTIL_H */
