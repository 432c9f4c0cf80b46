/*
 * lightgraph_scene.h -- seeded synthetic inputs for the LightGraph path.
 *
 * The reference renders OpenVDB files and EXR environment maps that are not
 * shipped with it (its scenes/ scripts point at /path/to/...). These host functions
 * build the stand-in inputs deterministically from a seed: fBm value-noise
 * volumes, interior point sets and a sky environment map. They have no
 * counterpart in the reference; the C ABI in lightgraph_c.h consumes their
 * output exactly as it would consume a loaded grid.
 *
 * All arithmetic is + - * / floor and sqrt (no libm transcendentals except in
 * lgs_envmap), compiled without FP contraction, so x86-64 and aarch64 hosts
 * produce bit-identical volumes and points.
 */
#ifndef LIGHTGRAPH_SCENE_H_
#define LIGHTGRAPH_SCENE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LGS_VOLUME_SPHERE_FBM  0  /* sphere r=0.4 of the unit box x fBm, clamped to [0,1] */
#define LGS_VOLUME_CUMULUS     1  /* cumulus puffs with a flat base, fBm-eroded, sparse   */
#define LGS_VOLUME_TEMPERATURE 2  /* fBm in [0, scale] wherever mask > 0                  */

/* Fills out[res^3] (x fastest) for a cube of res voxels (index range
 * [-res/2, res/2)). octaves: fBm octave count. scale multiplies the result
 * (1 for density, the maximum temperature for LGS_VOLUME_TEMPERATURE). mask is
 * only read for LGS_VOLUME_TEMPERATURE and may be null (then unmasked).
 * Returns the number of non-zero voxels. */
int64_t lgs_volume(int kind, int res, int octaves, uint64_t seed, double scale,
                   const float* mask, float* out);

/* Rejection-samples n points uniformly inside the active bbox of the grid
 * (res^3, index range [-res/2, res/2), world = index * voxel_size), keeping
 * those where the trilinear density is >= min_density (the reference's
 * PC_DENSITY_CUTOFF test, src/LightGraph.h:249). out: n x 3 floats.
 * Returns the number of points written (< n only if max_tries ran out). */
int64_t lgs_points(const float* density, int res, double voxel_size, int64_t n,
                   uint64_t seed, double min_density, int64_t max_tries, float* out);

/* Sky environment map, h rows x w cols x RGB floats (row 0 = zenith):
 * a zenith-to-horizon gradient, a dark ground, and a Gaussian sun lobe of
 * width sun_sigma_deg at elevation sun_elev_deg. Values are rounded to half
 * precision, as an EXR read through Imf::Rgba delivers them. */
void lgs_envmap(int w, int h, double sun_elev_deg, double sun_azim_deg,
                double sun_sigma_deg, double sun_intensity, float* out);

#ifdef __cplusplus
}
#endif

#endif /* LIGHTGRAPH_SCENE_H_ */
