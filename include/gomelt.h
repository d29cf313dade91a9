/*
 * gomelt.h -- C ABI of the GB300 (sm_103a) implementation of GO-MELT's
 * multilevel explicit thermal step.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*), enqueues work on that stream and returns a status code
 * (GM_OK = 0).  No entry point allocates device memory.  Floating-point
 * buffers are float (dtype GM_F32) or double (GM_F64), as the call says.
 *
 * Layout: every level is a structured node grid, node id = ix + iy*nx +
 * iz*nx*ny (x fastest), as in the reference's convert2XYZ
 * (go_melt/computeFunctions.py:645-689).  Phase bytes: bit0 = S1 (bulk),
 * bit1 = S2 (liquid).  Units are the reference's (mm, s, W, K).
 *
 * Each declaration names the reference function of GO-MELT
 * (JLnorthwestern/GO-MELT, go_melt/computeFunctions.py) that it replaces.
 */
#ifndef GOMELT_H
#define GOMELT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum gm_status_code {
  GM_OK = 0,
  GM_ERR_ARG = 1,         /* invalid argument (null pointer, size, dtype) */
  GM_ERR_LAUNCH = 2,      /* kernel launch failed */
  GM_ERR_CUDA = 3,        /* other CUDA runtime error */
  GM_ERR_UNSUPPORTED = 4, /* configuration the library does not handle */
  GM_ERR_TOO_LARGE = 5    /* request exceeds a fixed capacity */
};

enum gm_dtype { GM_F32 = 0, GM_F64 = 1 };

/* Material, laser and surface constants after the reference's set-up
 * (SetupProperties, computeFunctions.py:267-345).  Conductivities in W/(m K)
 * as in the input file (divided by 1000 inside), h_conv already multiplied by
 * 1e6 as the reference does (:318-319). */
typedef struct gm_props {
  double k_powder, k_bulk_a0, k_bulk_a1, k_fluid;
  double cp_solid_a0, cp_solid_a1, cp_mushy, cp_fluid, rho;
  double T_amb, T_solidus, T_liquidus, T_boiling;
  double h_conv, emissivity, sigma_sb, evc, Lev, CM_coeff, CT_coeff, CP_coeff;
  double laser_radius, laser_depth, laser_eta;
} gm_props;

/* Separable trilinear interpolation map from a source node grid to a tensor
 * grid of target points (interpolatePointsMatrix, :1028-1107).  Per axis d
 * and target index t: elem[d][t] = source element (clipped floor), w[d][2t]
 * = (x_{e+1} - x)/h, w[d][2t+1] = (x - x_e)/h (dtype of the call). */
typedef struct gm_map3 {
  int n[3];
  int src_nx, src_ny;
  const int* elem[3];
  const void* w[3];
} gm_map3;

/* One explicit level step, fused.  Replaces solveMatrixFreeFE (:582-642)
 * together with what the reference computes around it for one level:
 * computeStateProperties (:2567-2614), computeSourcesL3 (:2960-3012),
 * computeConvRadBC (:2207-2301), substitute_Tbar (:1848-1865), assignBCs
 * (:1568-1595) / assignBCsFine (:1598-1620) with the prolongated coarse field
 * (interpolate_w_matrix, :1110-1128), the T >= T_amb clamp and the melt-time
 * update (:3568-3578). */
typedef struct gm_level_args {
  int dtype;
  int nx, ny, nz;              /* nodes per axis */
  double h[3];                 /* node spacing */
  double origin[3];            /* coordinates of node 0 (for the laser source) */
  int ne_planes;               /* elements with ez < ne_planes are active */
  const double* dt;            /* device pointer: time step [s] */
  const void* T_in;            /* temperature at step start */
  void* T_out;                 /* new temperature (must not alias T_in) */
  const uint8_t* ph_in;        /* phase at step start (NULL: all zero) */
  uint8_t* ph_out;             /* updated phase (NULL: not written) */
  long long substrate;         /* nodes with id < substrate are always S1 */
  const void* k_arr;           /* optional nodal k [W/(mm K)]; NULL: from T/phase */
  const void* rc_arr;          /* optional nodal rho*cp; NULL: from T/phase */
  const void* F_full;          /* optional full-size RHS vector */
  const void* corr_full;       /* optional full-size correction vector */
  const void* rhs_box;         /* optional extra RHS on a node box */
  int box[6];                  /* box: x0,x1,y0,y1,z0,z1 (half-open) */
  const double* laser;         /* device laser row (x,y,z,...,P at [6]); NULL: no source */
  int surface;                 /* 1: conv/rad/evap flux on the top active plane */
  int bc_mode;                 /* 0: none, 1: constant faces, 2: prolongated coarse field,
                                  3: bc_new/bc_old are prolongated ring arrays of this level */
  double face[5];              /* bc_mode 1: x0, x1, y0, y1, z0 face values */
  int inactive_amb;            /* 1: nodes above the active region set to T_amb */
  const void* bc_new;          /* bc_mode 2: coarse field alpha*bc_new + beta*bc_old */
  const void* bc_old;
  double bc_alpha, bc_beta;
  gm_map3 bc_map;              /* coarse -> this level's nodes */
  int clamp;                   /* 1: T = max(T, T_amb) */
  void* accum;                 /* optional melt-time accumulators (Level 3): accum += dt at liquid nodes,
                                  reset when a node turns liquid, max_accum = running maximum of the
                                  reset values.  A node that is not liquid keeps its values (max_accum
                                  must be >= 0, as it starts at 0), so kernels may skip it. */
  void* max_accum;
  int zchunk;                  /* node planes per CTA (0: automatic) */
  int pdl;                     /* 1: the separable kernel may launch as a programmatic dependent of
                                  the preceding kernel in the stream (its CTAs start early and wait
                                  for that kernel before touching any field); dt and laser must not
                                  be written by that kernel.  0: ordinary stream order. */
  const void* src_tab;         /* optional: this step's laser factors from gm_fine_source_tables (one
                                  row); the separable kernel reads them instead of evaluating the
                                  Gaussians (with pdl, not written by the preceding kernels either) */
  int* status;                 /* optional device status word: a new value that is non-finite or above
                                  1e5 K (checked before the clamp; the bound of the reference's
                                  printLevelMaxMin, computeFunctions.py:3648-3658) sets GM_STATUS_BAD_T */
} gm_level_args;

int gm_level_step(const gm_level_args* a, const gm_props* p, void* stream);

/* Phase update and material properties per node (computeStateProperties,
 * :2567-2614): ph_out = (S1 | S2) from T and ph_in (S1 forced below
 * `substrate`); optional k [W/(mm K)] and rho*cp.  ph_out must not alias
 * ph_in. */
typedef struct gm_state_props_args {
  int dtype;
  long long n;
  const void* T;
  const uint8_t* ph_in;
  uint8_t* ph_out;
  void* k_out;
  void* rc_out;
  long long substrate;
} gm_state_props_args;

int gm_state_properties(const gm_state_props_args* a, const gm_props* p, void* stream);

/* Fine-level Gaussian source assembled on the nodes, added into F
 * (computeSourcesL3, :2960-3012).  laser: device row (x,y,z,...,P at [6]). */
int gm_fine_source(int dtype, const int nodes[3], const double origin[3], const double h[3], const double* laser,
                   const gm_props* p, void* F, void* stream);

/* Laser source factors of `nrows` fine steps on one window, tabulated once:
 * row i of `tab` (dtype, nrows x (nx + ny + nz)) holds the x factors times
 * the power factor, then the y and the z factors of laser row i (rows: 7
 * doubles each), as gm_level_step evaluates them (computeSourcesL3,
 * :2960-3012, separable form).  No counterpart in the reference. */
int gm_fine_source_tables(int dtype, const int nodes[3], const double origin[3], const double h[3],
                          const double* rows, int nrows, const gm_props* p, void* tab, void* stream);

/* Convection + radiation + evaporation flux of the top faces of element plane
 * ne_planes-1, added into F at node plane ne_planes (computeConvRadBC,
 * :2207-2301). */
int gm_surface_flux(int dtype, const int nodes[3], const double h[3], int ne_planes, const void* T, const gm_props* p,
                    void* F, void* stream);

/* Separable gather over a tensor grid of target points:
 *   out = base + sum_k coef[k] * I_k(src[k]),  k < nterms <= 3
 * and optionally out_term = I_which_term(src[which_term]).
 * Replaces interpolatePoints (:1131-1210) and interpolate_w_matrix
 * (:1110-1128); with base = fine T and coef = -1 it is the T' of
 * getNewTprime (:2097); with three terms it is the field remap of
 * moveEverything (:2427-2459). */
typedef struct gm_interp_args {
  int dtype;
  int n[3];
  int nterms;
  gm_map3 map[3];
  const void* src[3];
  double coef[3];
  const void* base; /* optional */
  void* out;
  void* out_term;   /* optional */
  int which_term;
} gm_interp_args;

int gm_interp(const gm_interp_args* a, void* stream);

/* Materialised interpolation matrix: Nc (npts x 8, dtype) and node (npts x 8)
 * for the target tensor grid of m (interpolatePointsMatrix, :1028-1107). */
int gm_interp_matrix(int dtype, const gm_map3* m, void* Nc, int* node, void* stream);

/* out[t] = sum_q Nc[t,q] * T[node[t,q]] (interpolate_w_matrix, :1110-1128). */
int gm_interp_w_matrix(int dtype, const void* Nc, const int* node, const void* T, void* out, long long n,
                       void* stream);

/* Restriction of getNewTprime (:2085-2093): coarse[cidx] = fine field
 * interpolated at the coarse overlap nodes (map: fine grid -> overlap
 * coordinates; cidx[d]: coarse node index of each overlap point per axis). */
typedef struct gm_restrict_args {
  int dtype;
  int n[3];
  gm_map3 map;
  const int* cidx[3];
  int cnx, cny;
  const void* fine;
  void* coarse;
} gm_restrict_args;

int gm_restrict(const gm_restrict_args* a, void* stream);

/* getNewTprime (:2060-2099) in ONE pass where the restriction is an
 * injection (every coarse overlap node coincides with a fine node, as on the
 * aligned level hierarchies): the coarse overlap nodes take the fine values
 * there, and T' = T_f - I(T_c) reads those values from the fine field, so
 * neither part waits for the other.  Per axis d and fine index f (length:
 * fine nodes along d): cf0[d][f] / cf1[d][f] = the fine index coinciding with
 * the low / high coarse node of f's coarse element (cmap) when that coarse
 * index is an overlap index, else -1; c_of_f[d][f] = the overlap coarse
 * index coinciding with f, else -1.  cmap: fine nodes -> coarse grid (the
 * prolongation map of gm_interp).  Equals gm_restrict + gm_interp with base =
 * fine, coef = -1 when the restriction weights are exactly 0 / 1.  No
 * counterpart in the reference (the two steps fused). */
typedef struct gm_tprime_args {
  int dtype;
  int n[3];              /* fine nodes */
  gm_map3 cmap;          /* fine nodes -> coarse grid */
  const int* cf0[3];
  const int* cf1[3];
  const int* c_of_f[3];
  int cnx, cny;          /* coarse node strides */
  const void* fine;      /* fine T */
  void* coarse;          /* coarse T: overlap nodes overwritten */
  void* out;             /* T' (fine nodes) */
} gm_tprime_args;

int gm_tprime_inject(const gm_tprime_args* a, void* stream);

/* Level-1 S1 from Level 2 (subcycleGOMELT :3272-3278, updateStateProperties
 * :2547-2556): S1 bit of coarse_ph at the overlap nodes := interpolated
 * Level-2 S1 > 0.499, or node id < substrate. */
typedef struct gm_restrict_s1_args {
  int dtype;
  int n[3];
  gm_map3 map;
  const int* cidx[3];
  int cnx, cny;
  const uint8_t* fine_ph;
  uint8_t* coarse_ph;
  long long substrate;
} gm_restrict_s1_args;

int gm_restrict_s1(const gm_restrict_s1_args* a, void* stream);

/* Level-0 phase store: S1 of every Level-0 node as one bit (the reference
 * keeps a float S1 and a bool S2 per node, computeFunctions.py:206-246; every
 * use of its S1 is S1 > 0.499).  Words of 32 bits, each (y, z) row of l0_nx
 * nodes padded to whole words: node (x, y, z) is bit x % 32 of word
 * (z * l0_ny + y) * ceil(l0_nx / 32) + x / 32 (gm_l0_words words in all).
 * gather: ph[t] = S1 from Level 0 at (idx[0][i], idx[1][j], idx[2][k]) plus
 *   the S2 bit of prev_ph where the previous window (Level-0 start prev_lo,
 *   size prev_n) covers the node (moveEverything :2500-2502; Level 0 keeps S2
 *   only inside the last scattered window, :2390-2392, :3628-3630).
 * scatter: Level-0 S1 at the window := S1 bit of ph (:2390-2391, :3628). */
typedef struct gm_l0_args {
  int n[3];
  const int* idx[3];
  long long l0_nx, l0_ny;
  uint32_t* l0_bits;
  uint8_t* ph;
  const uint8_t* prev_ph; /* gather only; NULL: no S2 anywhere */
  int prev_lo[3], prev_n[3];
} gm_l0_args;

/* Many level steps (windows of uneven sizes, e.g. independent scan
 * instances) in ONE launch: args[b] as for gm_level_step, props[b] per
 * instance; all with the same dtype and the same features (laser, RHS box,
 * bc_mode, melt time, ...).  desc: device buffer of at least
 * gm_level_batched_desc_size(nb, dtype) bytes for the per-instance
 * descriptors, rewritten in stream order by each call (the host side is
 * consumed before the call returns).  No counterpart in the reference. */
long long gm_level_batched_desc_size(int nb, int dtype);
int gm_level_step_batched(const gm_level_args* args, int nb, const gm_props* props, void* desc,
                          long long desc_bytes, void* stream);

/* The same in two parts: prepare (host -> desc, stream-ordered copies) and
 * launch (reads only desc: capturable in a CUDA graph and replayable while
 * desc is unchanged).  info receives what the launch needs. */
typedef struct gm_batch_info {
  int nb, dtype, variant, blocks;
  int kernel, rows, warps;  /* 1: separable kernel (constant-property batches), rows x warps a CTA */
} gm_batch_info;

int gm_level_batched_prepare(const gm_level_args* args, int nb, const gm_props* props, void* desc,
                             long long desc_bytes, gm_batch_info* info, void* stream);
int gm_level_batched_launch(const void* desc, const gm_batch_info* info, void* stream);

/* Launch shape of a level step.  kernel 0: element tiles, tile_x 32
 * (32 x 8 element columns a CTA) or 16 (16 x 16).  kernel 1: the separable
 * stencil for constant-property materials (constant k and rho*c; the
 * Level-1/2/3 feature sets of gm_subcycle, all nodes at or below the active
 * element planes unless inactive_amb): a warp owns 30 node columns (tile_x,
 * fixed) and `rows` (1, 2 or 4) y rows, tile_y (1..8) warps a CTA.
 * zchunk: node planes a CTA marches (at most 32 for kernel 1). */
typedef struct gm_level_shape {
  int kernel, tile_x, tile_y, rows, zchunk;
} gm_level_shape;

/* gm_level_step with an explicit launch shape (results agree with every
 * other shape to rounding; GM_ERR_ARG if the separable kernel is asked for a
 * call it does not serve).  No counterpart in the reference. */
int gm_level_step_shape(const gm_level_args* a, const gm_props* p, const gm_level_shape* shape, void* stream);

/* Autotuner: times gm_level_step for this call over the element tiles
 * (32 x 8, 16 x 16) and, where it applies, the separable kernel (1, 2 or 4
 * rows a thread, 2, 4 or 8 warps a CTA), each over the z-chunks (every distinct
 * split of the node planes), with CUDA events over a CUDA graph of 4*reps
 * back-to-back launches (programmatic dependents of one another, as
 * gm_subcycle issues them; issued directly on the legacy default stream) after
 * one untimed launch, and keeps the fastest for later calls with the same
 * dtype, features (melt time included) and grid that leave zchunk at 0.  The timed launches write
 * T_out / ph_out / melt time as the call would (so pass scratch outputs, or
 * tune a call whose repetition is harmless); synchronises the stream; not for
 * use during stream capture.  Result: the shape (fields as gm_level_shape;
 * for kernel 0 tile_y is the tile height and rows 1) and its time.
 * No counterpart in the reference. */
typedef struct gm_tune_result {
  int tile_x, tile_y, zchunk;
  float us;
  int kernel, rows;
} gm_tune_result;

int gm_level_autotune(const gm_level_args* a, const gm_props* p, int reps, gm_tune_result* out, void* stream);

/* Two consecutive Level-3 fine steps in ONE launch: the N3 inner steps of
 * computeSolutions_L3 within subcycleGOMELT's innermost lax.scan
 * (computeFunctions.py:3015-3054, :3404-3430, :3586-3622) taken two at a
 * time.  `level` is the first step (its dt, src_tab, bc_alpha / bc_beta)
 * and carries everything both steps share; dt2, src_tab2 and bc_alpha2 /
 * bc_beta2 are the second step's.  T_out, ph_out and the melt-time arrays
 * receive the fields after both steps, equal bit for bit to gm_level_step of
 * the first step followed by gm_level_step of the second on its output; the
 * intermediate fields are never written (the first step's values stay in the
 * kernel's registers).  Serves the constant-property Level-3 feature set:
 * laser factors from tables for both steps (src_tab and src_tab2 of
 * gm_fine_source_tables), surface flux, clamp, bc_mode 3 ring arrays, phase
 * in and out, optional melt time, ne_planes = nz - 1, nz >= 3; anything else
 * returns GM_ERR_UNSUPPORTED.  pdl as gm_level_step.  No counterpart in the
 * reference (which takes the steps one at a time). */
typedef struct gm_level2_args {
  gm_level_args level;
  const double* dt2;           /* device pointer: the second step's time step */
  const void* src_tab2;        /* the second step's laser factors (one gm_fine_source_tables row) */
  double bc_alpha2, bc_beta2;  /* the second step's ring blend */
} gm_level2_args;

int gm_level_step2(const gm_level2_args* a, const gm_props* p, void* stream);

/* gm_level_step2 with an explicit launch shape: kernel 2, rows (1, 2 or 4)
 * y rows a thread, tile_y (1..8) warps a CTA of 28 node columns each, zchunk
 * (1..30) output planes a CTA marches. */
int gm_level_step2_shape(const gm_level2_args* a, const gm_props* p, const gm_level_shape* shape, void* stream);

/* Autotuner of gm_level_step2 (as gm_level_autotune: CUDA-graph timing of
 * 4*reps back-to-back programmatic-dependent launches per candidate; writes
 * T_out / ph_out / melt time; synchronises; not during stream capture): the
 * fastest rows x warps x z-chunk is kept for later calls with the same dtype,
 * features and grid that leave zchunk at 0.  Result kernel = 2. */
int gm_level_autotune2(const gm_level2_args* a, const gm_props* p, int reps, gm_tune_result* out, void* stream);

/* Prolongation of one or two coarse fields onto the Dirichlet ring of a fine
 * level (faces x0, x1, y0, y1 and the bottom plane), written at the ring
 * nodes' ids in full-size arrays: outA = I(srcA), outB = I(srcB) (the
 * interpolate_w_matrix + assignBCsFine of computeL2Temperature :2937-2955 and
 * computeSolutions_L3 :3039-3052, with the coarse blend applied afterwards by
 * gm_level_step's bc_mode 3).  map: coarse grid -> fine nodes; srcB/outB
 * optional together. */
typedef struct gm_ring_args {
  int dtype;
  int nodes[3];
  gm_map3 map;
  const void* srcA;
  const void* srcB;
  void* outA;
  void* outB;
} gm_ring_args;

int gm_ring_prolong(const gm_ring_args* a, void* stream);

/* T = max(T, lo) over n values (the T >= T_amb clamp of stepGOMELT,
 * :2360-2362, :2380-2382). */
int gm_clamp_min(int dtype, void* T, long long n, double lo, void* stream);

int gm_l0_gather(const gm_l0_args* a, void* stream);
int gm_l0_scatter(const gm_l0_args* a, void* stream);
/* Words of the Level-0 store of an nx x ny x nz node grid (-1 if empty). */
long long gm_l0_words(long long nx, long long ny, long long nz);
/* Level-0 nodes [first, last) (node ids ix + iy nx + iz nx ny) set to value
 * (0 or 1): the substrate planes of a new layer (go_melt.py:198-314 via
 * getSubstrateNodes) and the planes freed by the layer shift (:258-296). */
int gm_l0_fill(uint32_t* l0_bits, long long nx, long long ny, long long nz, long long first, long long last, int value,
               void* stream);

/* Per-axis geometry of a fine level inside a coarse level, for the terms that
 * the reference evaluates through computeCoarseFineShapeFunctions
 * (:1213-1358).  For fine element e and Gauss side s (0: xi=-1/sqrt3,
 * 1: +1/sqrt3): cw[(e*2+s)*2 + A] = 1-D coarse weight of local coarse node A
 * (A=0: (x1-x)/H, A=1: (x-x0)/H) in the coarse element of that Gauss point;
 * node0[e] = coarse element of side 0 (whose nodes receive the result, as
 * the reference's BCOO does).  Coarse elements [cb_lo, cb_lo+ncb) receive
 * fine elements [flo[i], fhi[i]); rmax = max(fhi-flo); H = coarse spacing. */
typedef struct gm_couple_axis {
  int nfe;
  const void* cw;
  const int* node0;
  int cb_lo, ncb;
  const int* flo;
  const int* fhi;
  int rmax;
  double H;
} gm_couple_axis;

typedef struct gm_couple_geom {
  gm_couple_axis ax[3];
} gm_couple_geom;

/* Number of scratch elements (dtype) gm_couple needs for `partials` (enough
 * for either method). */
long long gm_couple_partials_size(const gm_couple_geom* g);

/* Fine -> coarse subgrid terms, added into `out` (a dtype array over the
 * coarse node box [out_lo, out_lo+out_n) per axis) times `scale`:
 *   Tp != NULL : flux term  -sum grad Nc . (kbar grad Tp) w
 *     (computeL1TprimeTerms_Part1 :2733-2810, computeL2TprimeTerms_Part1
 *      :2857-2914, computeCoarseTprimeTerm_jax :1477-1565)
 *   dTa != NULL: mass term  -sum Nc rcbar (dTa - dTb) w / dt
 *     (computeL1TprimeTerms_Part2 :3057-3132, computeL2TprimeTerms_Part2
 *      :3169-3221, computeCoarseTprimeMassTerm_jax :1396-1474)
 * kbar, rcbar: element means of k and rho*c from the fine T and phase
 * (computeStateProperties with `substrate`) or from k_arr/rc_arr.
 * `partials` is caller-provided scratch of partials_cap elements. */
typedef struct gm_couple_args {
  int dtype;
  gm_couple_geom geom;
  int fine_nodes[3];
  double fine_h[3];
  const void* T;
  const uint8_t* ph;
  long long substrate;
  const void* k_arr;
  const void* rc_arr;
  const void* Tp;
  const void* dTa;
  const void* dTb;
  const double* dt;
  void* out;
  int out_lo[3], out_n[3];
  double scale;
  void* partials;
  long long partials_cap;
  int method;  /* 0: separable contraction when k and rho*c are constant and the scratch holds it, else
                  the element reduction; 1: element reduction; 2: separable (constant properties only) */
  const void* base;  /* optional: out = base + scale * terms instead of out += (the output box must be
                        the coupling box: out_lo = cb_lo, out_n = ncb + 1; base must not alias out) */
} gm_couple_args;

int gm_couple(const gm_couple_args* a, const gm_props* p, void* stream);

/* Allocation-free form of gm_couple (this entry point has no counterpart in
 * the reference, which leaves all memory to JAX).  For callers that cannot
 * allocate device memory when they need the coupling terms -- e.g. code running
 * while another framework owns the device allocator, or a loop that must not
 * pay the synchronisation cudaMalloc/cudaFree may cause -- the partial sums
 * live in a library-owned __device__ array of GM_COUPLE_NOALLOC_SCRATCH_BYTES
 * (4 MiB: 1 Mi float or 512 Ki double partials), which every GPU that loads
 * the library keeps until exit.  Arguments are those of gm_couple; `partials`
 * and `partials_cap` are ignored.  The path is chosen as gm_couple chooses it
 * with a 4 MiB scratch: with method 0 and constant properties the separable
 * contraction when its partials fit, else the element reduction.  Returns
 * GM_ERR_TOO_LARGE when the path taken needs more partials than the array
 * holds.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture (a
 * first call on a stream that is being captured returns GM_ERR_ARG).
 * The array is shared by all calls and keeps the last call's contents; every
 * call overwrites all partials it reads, so nothing needs clearing, but calls
 * that overlap on the GPU (different streams, no ordering) race on it. */
#define GM_COUPLE_NOALLOC_SCRATCH_BYTES (4u << 20)
int gm_couple_noalloc(const gm_couple_args* a, const gm_props* p, void* stream);

/* Coarse laser source averaged over npos laser rows (computeLevelSource
 * :2667-2730; with npos = 1 the Fc/Fm of computeSources :928-988), added into
 * `out` (coarse node box as in gm_couple).  rows: device array of npos rows of
 * 7 doubles (x, y, z, ..., P at [6]); xq[d]: fine Gauss coordinates per axis
 * (nfe*2 doubles); fine_wq: fine quadrature weight hx*hy*hz/8; scratch:
 * npos*((ncb0+1)+(ncb1+1)+(ncb2+1)) dtype elements. */
typedef struct gm_coarse_source_args {
  int dtype;
  gm_couple_geom geom;
  int npos;
  const double* rows;
  const double* xq[3];
  double fine_wq;
  void* out;
  int out_lo[3], out_n[3];
  void* scratch;
  long long scratch_cap;
  /* ngroups > 1: the npos rows are ngroups consecutive groups of equal size,
   * each averaged into its own output box at out + g * out_group_stride
   * elements (one launch pair for several coarse steps); 0 or 1: one group. */
  int ngroups;
  long long out_group_stride;
} gm_coarse_source_args;

int gm_coarse_source(const gm_coarse_source_args* a, const gm_props* p, void* stream);

/* One level as the subcycle sees it: grid, state buffers and substrate count
 * (nodes with id < substrate are always S1, getSubstrateNodes :562-579). */
typedef struct gm_window {
  int nodes[3];
  double h[3];      /* node spacing */
  double origin[3]; /* node 0 coordinates */
  long long substrate;
  void* T;          /* temperature (state, dtype) */
  void* Tp;         /* subgrid field T' (Levels 2, 3) */
  uint8_t* ph;      /* phase bytes */
} gm_window;

/* Everything one subcycleGOMELT call (:3224-3632) needs: the three levels,
 * the per-window maps and coupling geometry of the current window positions,
 * the N2*N3 laser rows of the call, caller-provided work buffers (sizes in
 * elements of dtype unless noted) and optional per-Level-2-step histories. */
typedef struct gm_subcycle_plan {
  int dtype;
  int N2, N3;
  gm_window L1, L2, L3;
  int L1_ne_planes;          /* active Level-1 element planes (calcStaticTmpNodesAndElements) */
  double face[5];            /* Level-1 Dirichlet values: x0, x1, y0, y1, z0 */
  void* acc3;                /* melt time on the Level-3 window (accum_L3) */
  void* macc3;               /* its running maximum (max_accum_L3) */
  gm_map3 bc12, bc23;        /* Level 1 -> Level-2 nodes, Level 2 -> Level-3 nodes */
  gm_map3 r32, r21;          /* Level 3 at the Level-2 overlap nodes, Level 2 at the Level-1 overlap nodes */
  const int* r32_idx[3];     /* Level-2 node index of each Level-3 overlap point, per axis */
  const int* r21_idx[3];     /* Level-1 node index of each Level-2 overlap point, per axis */
  gm_couple_geom c32, c31, c21;
  const double* xq32[3];     /* Level-3 Gauss-point coordinates per axis (nfe*2) */
  const double* xq31[3];
  int rhs1_lo[3], rhs1_n[3]; /* Level-1 node box of the coupling terms (c21) */
  int rhs2_lo[3], rhs2_n[3]; /* Level-2 node box of the coupling terms (c32) */
  uint32_t* L0;              /* Level-0 S1 store, one bit a node (layout of gm_l0_args) */
  long long L0_nx, L0_ny;
  const int* l0_idx3[3];     /* Level-0 node index of the Level-3 window, per axis */
  const double* rows;        /* device: N2*N3 rows (x, y, z, jump, dwell, dt, P) */
  const double* dts;         /* device: N2+1 values: sum of all dt, then per Level-2 step */
  void* T1p;                 /* work: Level-1 predictor, corrector (nn1 each) */
  void* T1c;
  void* T2w[2];              /* work: nn2 each */
  void* T3w[2];              /* work: nn3 each */
  void* tp3w[2];             /* work: nn3 each */
  void* Tp2w;                /* work: nn2 */
  void* rhs1;                /* work: prod(rhs1_n) */
  void* rhs2;                /* work: prod(rhs2_n) */
  void* tp3hist;             /* work: N2*nn3 */
  uint8_t* ph2w[2];          /* work: nn2 bytes each */
  uint8_t* ph3w[2];          /* work: nn3 bytes each */
  void* partials;            /* scratch of gm_couple */
  long long partials_cap;
  void* src_scratch;         /* scratch of gm_coarse_source */
  long long src_cap;
  void* src2;                /* work: the N2 Level-2 source boxes of the call (N2 * rhs2 box values) */
  void* L2all;               /* optional (N2*nn2): Level-2 T after each corrector Level-2 step */
  void* L3all;               /* optional (N2*nn3): Level-3 T */
  void* L3pall;              /* optional (N2*nn3): Level-3 T' */
  int zchunk;                /* level-kernel tuning (0: automatic) */
  void* ring2[2];            /* work: Level-2 ring prolongations (nn2 each) */
  void* ring3[2];            /* work: Level-3 ring prolongations (nn3 each) */
  int graph;                 /* 1: capture the call's launches and run them as one CUDA graph, updated in
                                place from call to call on the same stream (the first call on a stream
                                issues directly) */
  int pdl;                   /* 1: every kernel of the call after the factor table launches as a
                                programmatic dependent of the kernel before it (its CTAs start while
                                that one drains and wait for it before touching any field) */
  void* src3tab;             /* optional work (N2*N3 * (nx+ny+nz) of Level 3): the Level-3 laser factors
                                of the call, tabulated at its start */
  int persist;               /* the N3 Level-3 steps of each Level-2 step as one launch (constant-property
                                materials with src3tab and the work below): 1 gm_level3_persist (window
                                in shared memory; a window without a persistent shape falls back to one
                                launch a step), 2 gm_level3_steps (grid barriers; pflags_cap >= 2 N2);
                                0: one launch a step */
  void* xch3[2];             /* work of persist: two nn3 fields (halo exchange) */
  unsigned* pflags;          /* work of persist: counters, zeroed by the call (mode 1: gm_level3_persist_flags(L3
                                nodes), mode 2: 2 N2) */
  long long pflags_cap;
  int* pstatus;              /* optional device status word: every level step of the call or-s
                                GM_STATUS_BAD_T into it for a non-finite or out-of-range new value, and
                                persist its GM_PERSIST_* bits (never cleared by the call; needed by
                                persist) */
  const int* inj32[9];       /* optional: cf0[3], cf1[3], c_of_f[3] of gm_tprime_inject for Level 3 ->
                                Level 2 when that restriction is an injection (its T' then takes one
                                launch) */
  const int* inj21[9];       /* the same for Level 2 -> Level 1 */
  int l3_pairs;              /* 1: the N3 Level-3 steps of a Level-2 step two at a time (gm_level_step2;
                                constant-property materials with src3tab, persist 0; an odd N3 ends
                                with one single step); 0: one launch a step */
} gm_subcycle_plan;

/* The whole subcycleGOMELT call (:3224-3632) enqueued on `stream`. */
int gm_subcycle(const gm_subcycle_plan* p, const gm_props* props, void* stream);

/* nb independent subcycleGOMELT calls (scan instances of uneven mesh sizes,
 * plans[i] with props[i]) as ONE CUDA graph launched on `stream` (not the
 * legacy default stream): instance i is issued on a branch stream forked from
 * `stream` and joined back, so the instances run concurrently.  The graph of
 * a stream and batch size is updated in place from call to call (same
 * topology while the instances keep their feature sets); the first call of a
 * batch issues the branches directly.  Plans must not ask for the persistent
 * Level-3 kernel (concurrent cooperative launches are not co-scheduled).
 * Results are those of nb gm_subcycle calls.  No counterpart in the reference
 * (which runs one instance a process). */
int gm_subcycle_batched(const gm_subcycle_plan* plans, int nb, const gm_props* props, void* stream);

/* ------------------------------------------------------------------------
 * The N3 Level-3 fine steps of one Level-2 step in ONE launch (persistent
 * kernel).  Replaces the inner lax.scan of subcycleGOMELT
 * (go_melt/computeFunctions.py:3404-3430 predictor, :3586-3622 corrector):
 * per step computeStateProperties, computeSourcesL3, computeConvRadBC,
 * computeSolutions_L3 with the blended Level-2 ring, the T >= T_amb clamp and,
 * with accumulators, the melt-time update (:3568-3578) -- the same arithmetic
 * as gm_level_step's separable kernel with bc_mode 3 and a laser factor table,
 * bit for bit.  Constant-property materials, every element plane active.
 * Step s blends the ring as alpha = (s+1)/nsub, beta = 1 - alpha.
 *
 * One cooperative launch keeps the window in shared memory (a tile of node
 * columns per CTA) and exchanges tile edges through `xbuf` between steps,
 * synchronised by per-tile counters in `flags`: every flag must equal `base`
 * when the launch starts and equals base + nsteps after it completes (zero
 * the flags once, then pass base += nsteps from launch to launch).  Waits are
 * bounded (about one second): a timeout sets GM_PERSIST_TIMEOUT in *status
 * and the launch ends with T_out incomplete (zero the flags again before the
 * next launch).  A final field with a non-finite value or a value above 1e5 K
 * sets GM_PERSIST_BAD_T.  GM_ERR_UNSUPPORTED when the window's tiles cannot
 * all be resident at once (the caller then issues gm_level_step per step).
 * No counterpart in the reference.
 * ------------------------------------------------------------------------ */
#define GM_PERSIST_TIMEOUT 1
#define GM_PERSIST_BAD_T 2
#define GM_STATUS_BAD_T GM_PERSIST_BAD_T /* level steps: gm_level_args.status */

typedef struct gm_persist_args {
  int dtype;
  int nodes[3];
  double h[3];
  int nsteps;                  /* fine steps of this launch */
  int nsub;                    /* ring blend denominator (N3) */
  const void* T_in;            /* window at the first step's start */
  void* T_out;                 /* window after the last step (may be xbuf[nsteps % 2], not T_in) */
  const uint8_t* ph_in;
  uint8_t* ph_out;
  long long substrate;         /* nodes with id < substrate are always S1 */
  const void* ring_new;        /* coarse field at the step's end, prolongated onto the ring nodes */
  const void* ring_old;        /* coarse field at the step's start, likewise (gm_ring_prolong) */
  const void* src_tab;         /* nsteps rows of laser factors (gm_fine_source_tables) */
  const double* rows;          /* nsteps toolpath rows (x, y, z, jump, dwell, dt, P) */
  void* accum;                 /* optional melt-time accumulators (both or neither) */
  void* max_accum;
  void* xbuf[2];               /* work: two full-size fields, neither aliasing T_in */
  unsigned* flags;             /* work: per-tile step counters (gm_level3_persist_flags) */
  long long flags_cap;
  unsigned base;               /* value of every flag when the launch starts */
  int* status;                 /* device word: GM_PERSIST_* bits are or-ed into it */
  int hold;                    /* 0 in every ordinary call.  t > 0: tile t-1 withholds its step counters
                                  (failure injection for tests: its neighbours' waits run out) */
} gm_persist_args;

/* Number of flags (tiles) of a window, or -1 if the window has no persistent
 * shape; the flag array of a call must hold at least this many. */
long long gm_level3_persist_flags(const int nodes[3]);
/* Tile shape of a window: out = {tiles, x columns a tile, y rows a tile, z
 * segments a tile row}; GM_ERR_UNSUPPORTED if the window has none. */
int gm_level3_persist_shape(int dtype, const int nodes[3], int out[4]);
int gm_level3_persist(const gm_persist_args* a, const gm_props* p, void* stream);

/* ------------------------------------------------------------------------
 * Toolpath rows on the device, positions and time accumulated in FP64.
 * Replaces the text round trip of the reference (createPath.py:126-160
 * writes x += vx*dt per fine step as %.8e text; go_melt.py:140-160 reads N2*N3
 * lines a chunk).  `runs` (device, nruns x 11 doubles: kind, count, x, y, z,
 * jump, ux, uy, dt, P, short; kind 0 = move: position set to (x, y), count
 * rows after x += ux*dt, y += uy*dt, then one row after += u*short if short
 * > 0; kind 1 = hold: count rows at (x, y), dwell flag 0, power 0) is built
 * by createPath.toolpath_runs.  Each call writes the next `nrows` rows
 * (x, y, z, jump, dwell, dt, P) and dts = {sum of their dt, then the sum of
 * each of `ngroups` equal groups}, sums in row order; rows past the end of the
 * table are zero.  Products are rounded before the sums (no fused
 * multiply-add), so the rows equal the host's float64 ones bit for bit.
 * *state (device, zeroed before the first call) carries the cursor, the
 * position and the elapsed time t between calls.  No counterpart in the
 * reference (its accumulation is host Python).
 * ------------------------------------------------------------------------ */
typedef struct gm_toolpath_state {
  long long run, k;  /* run index and rows emitted of it */
  long long row;     /* rows emitted in all */
  double x, y;       /* position of the current move */
  double t;          /* elapsed time: sum of the emitted rows' dt */
} gm_toolpath_state;

int gm_toolpath_rows(const double* runs, int nruns, gm_toolpath_state* state, int nrows, int ngroups, double* rows,
                     double* dts, void* stream);

/* The N3 Level-3 steps of one Level-2 step in ONE cooperative launch, every
 * step the separable one-step kernel's arithmetic over its tiles (results are
 * gm_level_step's, bit for bit: the same inner lax.scan of subcycleGOMELT,
 * computeFunctions.py:3404-3430, :3586-3622, as gm_level3_persist), the
 * fields staying in L2 between steps and a grid barrier on `counter` between
 * them.  `level` is one step's gm_level_args (bc_mode 3 ring arrays, phase
 * in and out, optional melt time, laser set); T_in is the first step's input
 * and T_out the last step's output; step s reads rows + 7 s (dt at [5]) and
 * laser factor row s of src_tab and blends the ring with alpha = (s+1)/nsub.
 * tbuf: two work fields aliasing neither T_in nor T_out.  `counter` must
 * equal `base` when the launch starts (the launch leaves it at base +
 * (nsteps - 1) x its grid size: give every launch its own zeroed counter).
 * Barrier waits are bounded (about one second, GM_PERSIST_TIMEOUT in
 * *status).  Constant-property materials; GM_ERR_UNSUPPORTED otherwise.  No
 * counterpart in the reference. */
typedef struct gm_steps_args {
  gm_level_args level;
  int nsteps, nsub;
  const double* rows;
  const void* src_tab;
  void* tbuf[2];
  unsigned* counter;
  unsigned base;
  int* status;
} gm_steps_args;

int gm_level3_steps(const gm_steps_args* a, const gm_props* p, void* stream);

/* Library identification: returns a static string; never fails. */
const char* gm_version(void);

/* ------------------------------------------------------------------------
 * Diagnostics (no counterpart in the reference; quantities the GB300 build
 * reports beside its results).  All reduce in FP64 with two-stage,
 * fixed-order reductions, and write their results to device memory (`out`).
 * `scratch` holds gm_diag_scratch_size(npos) doubles of device memory.
 * ------------------------------------------------------------------------ */
long long gm_diag_scratch_size(int npos);

/* Energy balance of a level window over an interval [t0, t0 + interval]
 * from its fields at both ends (T0, T1) and the laser rows of the fine steps
 * in between.  With interior nodes I = {1 <= ix <= nx-2, 1 <= iy <= ny-2,
 * 1 <= iz <= ne_planes} (the nodes not on the Dirichlet ring),
 * T_bar = (T0 + T1) / 2 and properties from T_bar and the phase ph of t0:
 *   out[0] stored  = sum_{i in I} V_i (h(T1_i) - h(T0_i)),  V_i = sum_e wq
 *                    (lumped volume), h(T) = rho * integral of c_p(T) dT of
 *                    the phase model (c1 T + c0 below T_solidus, c_mushy up
 *                    to T_liquidus, c_fluid above)
 *   out[1] source  = sum_rows dt_r sum_{i in I} F_src,i(row r)
 *   out[2] surface = interval * sum_{i in I} F_surf,i(T_bar)
 *   out[3] conduct = -interval * sum_{i in I} (K(T_bar) T_bar)_i
 * with the lumped mass, stiffness, laser source and surface flux of
 * solveMatrixFreeFE / computeSourcesL3 / computeConvRadBC.  The residual
 * |out[0] - out[1] - out[2] - out[3]| / (eta * sum_r dt_r P_r) is the
 * relative energy-balance error that accepts or rejects a predicted field. */
typedef struct gm_energy_args {
  int dtype; /* of T0 and T1 */
  int nodes[3];
  double h[3];
  double origin[3];
  int ne_planes;
  const void* T0;
  const void* T1;
  const uint8_t* ph; /* phase byte at t0 (may be NULL: powder) */
  long long substrate;
  double interval;
  const double* rows; /* npos laser rows (x, y, z, -, -, dt, P) */
  int npos;
  double* scratch;
  long long scratch_cap; /* doubles */
  double* out;           /* 4 doubles */
} gm_energy_args;

int gm_energy_balance(const gm_energy_args* a, const gm_props* p, void* stream);

/* Melt-pool extent at the isotherm T = iso: over the nodes with T >= iso,
 * the min / max coordinate per axis, each extended to the linearly
 * interpolated crossing towards every neighbour with T < iso.
 * out = {xmin, xmax, ymin, ymax, zmin, zmax, count}; count 0 leaves the
 * extents at +-inf.  Length / width / depth = xmax-xmin, ymax-ymin,
 * z_top-zmin. */
typedef struct gm_meltpool_args {
  int dtype;
  int nodes[3];
  double h[3];
  double origin[3];
  const void* T;
  double iso;
  double* scratch;
  long long scratch_cap; /* doubles */
  double* out;           /* 7 doubles */
} gm_meltpool_args;

int gm_melt_pool(const gm_meltpool_args* a, void* stream);

/* out = {max |A - B|, sqrt(mean (A - B)^2)} over n values (A, B of types
 * dtype_a, dtype_b: e.g. an FP32 run against an FP64 run). */
int gm_field_error(int dtype_a, const void* A, int dtype_b, const void* B, long long n, double* scratch,
                   long long scratch_cap, double* out, void* stream);

/* ------------------------------------------------------------------------
 * Level-3 surrogate (no counterpart in the reference): BF16 tensor-core
 * building blocks of a 3-D convolutional U-Net, trained and run on the
 * device.  Activations are channels-last BF16 [B][Z][Y][X][C]; a tensor
 * argument is a channel slice (offset, stride) of a wider tensor.  grid =
 * {B, X, Y, Z}.  3x3x3 weights are BF16 [27][Cout][Cin] (tap = dx + 3 dy +
 * 9 dz for offsets dx-1, dy-1, dz-1), zero padding at the sample borders.
 * ------------------------------------------------------------------------ */
typedef struct gm_conv_args {
  int grid[4];
  int cin, cout;         /* cin % 16 == 0; cout in {16, 32, 64, 96, 128, 192} */
  const void* in;        /* BF16 */
  int in_stride, in_off; /* even */
  const void* w;         /* BF16 [27][cout][cin] */
  const float* bias;     /* [cout] or NULL */
  int relu;              /* y = max(y, 0) */
  const void* mask;      /* BF16 or NULL: y = 0 where mask <= 0 */
  int mask_stride, mask_off;
  int mirror;            /* 1: tap offsets negated (data gradient with W^T) */
  void* out;             /* BF16 */
  int out_stride, out_off;
  void* wpack;           /* optional work of the tensor-core form (27 cin cout BF16): the weights are
                            repacked into it once per call in the layout of its shared-memory weight
                            tiles, so each tile arrives as one contiguous bulk copy; NULL: the tiles are
                            gathered from w by tensor copies of 16-byte rows */
} gm_conv_args;

/* y[v][co] = act(bias[co] + sum_tap sum_ci x[v + d(tap)][ci] w[tap][co][ci])
 * (mirror 0), or the data gradient dx[u][ci] = sum_tap dy[u - d(tap)] .
 * w[tap][.][ci] with w passed as [27][Cin][Cout] (mirror 1). */
int gm_unet_conv3(const gm_conv_args* a, void* stream);

/* The two forms gm_unet_conv3 chooses between.  _tc: tcgen05.mma (BF16 in,
 * FP32 accumulators in tensor memory), operand tiles by TMA
 * (cp.async.bulk.tensor, zero fill at the sample borders); needs cin and cout
 * multiples of 16 with cout <= 256, and 16-byte aligned bases and slices
 * (in/out/mask offsets and strides multiples of 8); GM_ERR_UNSUPPORTED
 * otherwise.  _mma: the warp-level mma.sync.m16n8k16 form (any even slice).
 * gm_unet_conv3 takes _tc when gm_unet_conv3_tc_eligible(a) returns 1. */
int gm_unet_conv3_tc(const gm_conv_args* a, void* stream);
int gm_unet_conv3_mma(const gm_conv_args* a, void* stream);
int gm_unet_conv3_tc_eligible(const gm_conv_args* a);
/* Waits of the tensor-core convolutions that ran out since the last call
 * (bit 0), -1 on a CUDA error; clears the word; synchronises the device. */
int gm_unet_tc_status(void);

typedef struct gm_wgrad_args {
  int grid[4];
  int cin, cout; /* cin % 32 == 0 or cin == 16; cout % 16 == 0 */
  const void* in;
  int in_stride, in_off;
  const void* dy;
  int dy_stride, dy_off;
  float* dw;     /* FP32 [27][cout][cin] */
  float* scratch;
  long long scratch_cap; /* floats: gm_unet_wgrad_scratch() */
} gm_wgrad_args;

/* dw[tap][co][ci] = sum_v dy[v][co] x[v + d(tap)][ci] (split over the
 * voxels, partials summed in a fixed order). */
long long gm_unet_wgrad_scratch(const int grid[4], int cin, int cout);
int gm_unet_wgrad(const gm_wgrad_args* a, void* stream);

/* db[c] = sum_v dy[v][c]; scratch: ceil(V / 4096) * C floats (at most 1024 * C). */
int gm_unet_bias_grad(const int grid[4], int C, const void* dy, int stride, int off, float* scratch,
                      long long scratch_cap, float* db, void* stream);

/* 2x average pooling of grid (forward: out on grid / 2) or its gradient
 * (backward: in on grid / 2, out on grid). */
int gm_unet_pool2(const int grid[4], int C, const void* in, int in_stride, int in_off, void* out, int out_stride,
                  int out_off, int backward, void* stream);

/* 2x nearest upsampling onto grid (forward: in on grid / 2) or its gradient
 * (backward: in on grid, out on grid / 2). */
int gm_unet_up2(const int grid[4], int C, const void* in, int in_stride, int in_off, void* out, int out_stride,
                int out_off, int backward, void* stream);

/* b[v][c] += a[v][c] over V voxels and C channels (BF16 slices), where
 * mask[v][c] > 0 if a mask slice is given. */
int gm_unet_add_slice(long long V, int C, const void* a, int a_stride, int a_off, void* b, int b_stride, int b_off,
                      const void* mask, int mask_stride, int mask_off, void* stream);

/* Head: out[v] = b + sum_c w[c] x[v][c] (FP32 out), and its backward for the
 * loss mean over voxels of lmask (pred - target)^2 (inv_count = 1 / sum lmask):
 * dx (zero where x <= 0, the head's input being a ReLU output) and
 * dwb = {dw[0..C), db, loss}.  C <= 32. */
int gm_unet_head(long long V, int C, const void* in, int in_stride, int in_off, const float* w, float b, float* out,
                 void* stream);
long long gm_unet_head_scratch(long long V, int C);
int gm_unet_head_bwd(long long V, int C, const void* in, int in_stride, int in_off, const float* w, const float* pred,
                     const float* target, const float* lmask, float inv_count, void* dx, int dx_stride, int dx_off,
                     float* scratch, long long scratch_cap, float* dwb, void* stream);

/* Adam step on an FP32 master copy w (n values) with gradient grad, moments
 * m, v; c1 = 1 - beta1^t, c2 = 1 - beta2^t; wd: L2 weight decay.  Writes the
 * BF16 copy wb and, if wt is set, its [27][cin][cout] transpose. */
typedef struct gm_adam_args {
  long long n;
  float* w;
  const float* grad;
  float* m;
  float* v;
  float lr, beta1, beta2, eps, c1, c2, wd;
  void* wb;
  void* wt;
  int cout, cin;
} gm_adam_args;

int gm_unet_adam(const gm_adam_args* a, void* stream);

/* Surrogate input / output on B windows of `nodes` nodes each (FP32 fields,
 * sample b at offset b * nodes[0] * nodes[1] * nodes[2]).  The network grid
 * {B, X, Y, Z} covers the nodes ix < X, iy < Y, 1 <= iz <= Z.  x: BF16
 * [V][16] channels (I(T2) - T_amb) / S, (T3_start - T_amb) / S, node offset
 * from the mid-step laser position (x, y) * inv_r, P / P_s, v / v_s, zeros;
 * target = (T3_end - I(T2)) / S (if T3n and target are set); lmask = 1 off
 * the Dirichlet ring (ix, iy >= 1).  par: 8 doubles per sample: window
 * origin x, y, spacing h, laser x, y, inv_r, P / P_s, v / v_s.  Unpack:
 * T3 = I(T2) + S * pred on the grid's nodes off the ring. */
typedef struct gm_surr_args {
  int grid[4];
  int nodes[3];
  const float* T2i;
  const float* T3o;
  const float* T3n;
  const double* par;
  double T_amb, scale;
  void* x;
  float* target;
  float* lmask;
} gm_surr_args;

int gm_surrogate_pack(const gm_surr_args* a, void* stream);
int gm_surrogate_unpack(const gm_surr_args* a, const float* pred, float* T3, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GOMELT_H */
