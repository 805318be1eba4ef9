/*
 * oracle.h — CPU restatement of YetAnotherSLAM's dense RGB-D path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker the parity tests,
 * the smoke test and the CPU-baseline leg of the benchmark compare the CUDA
 * path against; the product never links, loads or calls it.
 *
 * Parity status: the reference's dense path cannot be compiled here (it
 * needs OpenCV with CUDA modules, Eigen and Sophus, none of which is
 * installed) and its repository ships no tests or golden vectors for this
 * path.  The one piece of reference data on the path, its marching-cubes
 * table (RGBDFusion/utils/TriangleTable.h), pins this restatement's table
 * generator (edge masks, triangle counts and oriented polygons of every
 * case; tests/test_mc_reference_topology.py).  Everything else is pinned by
 * the analytic known-answer tests under tests/ (plane and sphere TSDFs,
 * exact plane raycasts, sphere meshes, known-motion recovery), not by
 * outputs of the reference itself.
 *
 * Precision: every discrete decision the reference makes from FP32 geometry
 * (block allocation along each ray, block visibility, the pixel a voxel
 * projects to, the truncation gate, z-range tile coverage; in the tracker,
 * the reference pixels that project inside the current image, the ICP
 * pairs and gates at the FP32 pose, and GetTransform's FP32 error and its
 * keep-the-better-estimate comparison) is evaluated in IEEE FP32 with one
 * rounding per operation in a fixed order (build with -ffp-contract=off),
 * exactly as the CUDA path does; continuous quantities
 * (TSDF accumulation, ray marching, image pyramids, residuals, reductions,
 * the 6x6 solve and the SE(3) update) use `real`, which is double in the
 * checker build (liboracle64) and float in the multi-threaded CPU-baseline
 * build (liboracle32).
 *
 * Reference files cited as path:line relative to the reference project root.
 */
#ifndef YAS_ORACLE_H
#define YAS_ORACLE_H

#include <stdint.h>

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif
typedef ORACLE_REAL real;

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ map */
typedef struct orc_map orc_map;

orc_map *orc_map_create(float voxel_size, float trunc, float depth_min, float depth_max, int max_weight);
/* 1: every written sdf goes through the reference's int16 storage. */
void orc_map_set_storage(orc_map *m, int int16_sdf);
void orc_map_destroy(orc_map *m);
int orc_map_num_blocks(const orc_map *m);
/* Allocation only (CreateBlockLineTracingFunctor). K = {fx, fy, cx, cy}. */
void orc_map_allocate(orc_map *m, const float *depth, int w, int h, const float *K, const double *Tcm);
/* Visible blocks at Tcm for a cols x rows image; writes up to cap coords. */
int orc_map_visible(orc_map *m, int cols, int rows, const float *K, const double *Tcm, int *coords, int cap);
/* Fuse(depth, Tcm): allocation + visibility + integration; returns #visible. */
int orc_map_fuse(orc_map *m, const float *depth, int w, int h, const float *K, const double *Tcm);
/* De-integration of one depth frame (the inverse running-average update). */
int orc_map_defuse(orc_map *m, const float *depth, int w, int h, const float *K, const double *Tcm);
/* MapStruct::Fuse(MapStruct*): fuses src into dst (poses: 3x4 world poses of
 * the two submaps); returns 1 if dst was empty and took src's storage. */
int orc_map_fuse_map(orc_map *dst, orc_map *src, const double *Tdst, const double *Tsrc);
/* Block coords (3 ints), sdf and weight (512 each) in insertion order. */
void orc_map_export(const orc_map *m, int *coords, double *sdf, double *wt);
/* Inserts/overwrites blocks with given float contents. */
void orc_map_import(orc_map *m, const int *coords, const float *sdf, const float *wt, int n);
/* Raycast at Tcm: vmap (w*h*4 floats, camera frame, w=+1 hit / -1 miss),
 * znear/zfar ((w+7)/8 * (h+7)/8) may be NULL. */
void orc_raycast(orc_map *m, int w, int h, const float *K, const double *Tcm, float *vmap, float *znear, float *zfar);
/* Marching cubes over all blocks: tris 9 floats each, cases, cube_xyz; returns
 * the number of triangles (writes at most cap). */
/* RenderScene: Phong shading of a vertex/normal map (float4, w*h) into RGBA8. */
void orc_render_scene(const float *vmap, const float *nmap, int w, int h, const float *light, unsigned char *rgba);
void orc_canvas_draw(const float *pts, const float *nrm, unsigned ntris, const double *Tmw, const double *Tcw,
                     const float *K4, int w, int h, uint64_t *keys);
int orc_mesh(const orc_map *m, float *tris, float *normals, int *cases, int *cube_xyz, int cap);
void orc_mc_tables(unsigned short *edge, signed char *tri, unsigned char *count);

/* ------------------------------------------------------------ tracker */
typedef struct orc_tracker orc_tracker;

orc_tracker *orc_tracker_create(int w, int h, const double *K, int levels, const int *iters, int mode);
void orc_tracker_destroy(orc_tracker *t);
void orc_tracker_set_image(orc_tracker *t, const uint8_t *gray, int reference);
void orc_tracker_set_depth(orc_tracker *t, const float *depth, int reference);
void orc_tracker_set_model(orc_tracker *t, const float *vmap);
void orc_tracker_swap(orc_tracker *t);
/* Returns 0, or 6 (NaN in the solve; out = identity). */
int orc_tracker_get_transform(orc_tracker *t, const double *init, int swap, double *out);
void orc_tracker_compute_step(orc_tracker *t, int level, const double *T, double *H, double *b, double *stats);
/* Copies a pyramid buffer as floats (which: as yas_tracker_level_buffer). */
void orc_tracker_level(const orc_tracker *t, int level, int which, float *out);

/* ------------------------------------------------------------ session */
typedef struct orc_session orc_session;

orc_session *orc_session_create(int w, int h, const float *K, float voxel_size, float trunc, int levels,
                                const int *iters, int mode, float depth_scale, float max_step);
void orc_session_destroy(orc_session *s);
/* rgb: w*h*3 uint8, depth: w*h uint16; out_Tcm row-major 3x4; returns status. */
int orc_session_frame(orc_session *s, const uint8_t *rgb, const uint16_t *depth, double *out_Tcm);
orc_map *orc_session_map(orc_session *s);
orc_tracker *orc_session_tracker(orc_session *s);

/* ------------------------------------------------------------ utilities */
void orc_se3_exp(const double *xi, double *T);
void orc_ldlt_solve6(const double *A, const double *b, double *x);
int orc_real_bytes(void);

#ifdef __cplusplus
}
#endif
#endif
