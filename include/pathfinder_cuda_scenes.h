/*
 * pathfinder_cuda_scenes.h — seeded synthetic scenes for tests and benchmarks.
 *
 * These entry points have no counterpart in the reference: the reference's
 * benchmarks load SVG files through usvg and fonts through font-kit, neither of
 * which is part of the rendering path.  The generators build scenes with the
 * shapes, sizes and value distributions of the workloads the CUDA level is
 * measured on, deterministically from a 64-bit seed (std::mt19937_64 with
 * this library's own uniform/normal transforms, so that every machine gets
 * the same bytes).
 */
#ifndef PATHFINDER_CUDA_SCENES_H
#define PATHFINDER_CUDA_SCENES_H

#include "pathfinder_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Workloads. */
#define PF_SCENE_STARS_512      1  /* 64 star paths, 8-32 quad/cubic edges, 512x512, nonzero, opaque   */
#define PF_SCENE_SVG_4K         2  /* 20,000 paths, ~2.1M segments, 3840x2160, mixed rules/alpha/clips */
#define PF_SCENE_GLYPH_ATLAS    3  /* 16,384 synthetic glyphs shelf-packed into a 4096x4096 atlas       */
#define PF_SCENE_CUBIC_1K       4  /* 256 closed cubic paths, 4,096 control points, 1024x1024           */
#define PF_SCENE_EDGE_CASES     5  /* small hand-built cases: tile corners, edges, above-view paths     */

typedef struct PFCUDASceneBuffers* PFCUDASceneBuffersRef;

/* Parameters.  `scale` in (0, 1] shrinks the path count of a workload (for
 * small parity cases); 1.0 is the full workload.  `jitter_sigma` perturbs
 * every point with N(0, sigma) px after generation (0 = none; the
 * differentiable target uses 2.0). */
typedef struct PFCUDASceneParams {
    int32_t  workload;
    uint64_t seed;
    double   scale;
    double   jitter_sigma;
    uint64_t jitter_seed;
    int32_t  width, height;   /* 0: the workload's own canvas */
} PFCUDASceneParams;

int32_t PFCUDASceneGenerate(const PFCUDASceneParams* params, PFCUDASceneBuffersRef* out);
/* Host-memory description of the generated scene (valid until Destroy). */
int32_t PFCUDASceneGetDesc(PFCUDASceneBuffersRef scene, PFCUDASceneDesc* out_desc,
                           int32_t* out_width, int32_t* out_height);
/* Glyph atlas only: per glyph its cell in the atlas (x0, y0, x1, y1). */
int32_t PFCUDASceneGetCells(PFCUDASceneBuffersRef scene, PFRectI* cells, uint32_t capacity);
int32_t PFCUDASceneDestroy(PFCUDASceneBuffersRef scene);

#ifdef __cplusplus
}
#endif
#endif
