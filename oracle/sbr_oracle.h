/* C interface of the CPU restatement (TEST INFRASTRUCTURE: the oracle).
 * Only tests, the smoke check and the benchmark's CPU-baseline leg call it. */
#ifndef SBR_ORACLE_H
#define SBR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* MaterialProperties field order (SBRSolver_rev2/common/DataStructures.h:20-28),
 * then the wall thickness passed to the slab coefficients (the reference
 * passes 0, FieldCompute.cpp:131,138). */
typedef struct {
  double frequency, transmissionLoss, reflectionLoss, relPermittivityRe, relPermittivityIm,
      relConductivity, width;
} MaterialProperties_c;

/* Arguments of RTSolver::ExecuteRayTracing (SBRSolver_rev2/RTSolver.h:25-37)
 * plus the antenna type FieldCompute.cpp:117 hard-codes (1). */
typedef struct {
  double tx[3];
  double tx_coord_sys[9]; /* row-major */
  int max_reflection, max_transmission;
  double frequency, pt;
  int use_fresnel;
  int tessellation;
  int antenna;
  int n_rx;
  const double* rx; /* 3 per receiver */
  int n_materials;
  const MaterialProperties_c* materials;
  /* antenna 3 (tabulated): the TXPattern.dat grid (data/TXPattern.dat, read
   * by Preprocessor::ReadPatternFile, Preprocessor.cpp:3-35) as
   * pat_nt x pat_np rows of (g_theta dB, arg_theta deg, g_phi dB, arg_phi deg),
   * theta-major, steps pat_dt / pat_dp degrees from theta = phi = 0. */
  const float* pattern;
  int pat_nt, pat_np;
  double pat_dt, pat_dp;
} oracle_request;

typedef struct {
  int receiver;
  int n_rays;
  long launch;
  double field[6]; /* this path's contribution: Ex re, im, Ey re, im, Ez re, im */
} oracle_path;

typedef struct oracle_scene oracle_scene;
typedef struct oracle_result oracle_result;

int oracle_scene_from_stl(const char* path, oracle_scene** out);
int oracle_scene_from_triangles(int n, const float* v, const float* normals, oracle_scene** out);
int oracle_scene_set_materials(oracle_scene* sc, const int* mat_ids);
int oracle_scene_info(const oracle_scene* sc, int* n_tri, int* n_nodes);
int oracle_scene_mesh_order(const oracle_scene* sc, int* out);
int oracle_scene_coplanar(const oracle_scene* sc, int* out);
void oracle_scene_destroy(oracle_scene* sc);
int oracle_icosphere(int level, double* out, long cap);
int oracle_solve(const oracle_scene* sc, const oracle_request* rq, int threads,
                 oracle_result** out);
void oracle_result_counts(const oracle_result* r, long* segments, long* captured,
                          long* corrected, long* n_paths, long* n_rays);
void oracle_result_copy(const oracle_result* r, double* field, oracle_path* paths,
                        long* ray_offset, int* tri, int* cop, int* kind, double* pts);
void oracle_result_destroy(oracle_result* r);

#ifdef __cplusplus
}
#endif
#endif
