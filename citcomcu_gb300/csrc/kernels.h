// Launchers for the sm_103a kernels of the Stokes / SUPG hot path.
// Every launcher enqueues on `st` and returns immediately; none allocates.
#pragma once

#include <cuda_runtime.h>

#include "level.h"

// Geometry of one element (device resident): one entry per level for the
// box, one per (theta, r) column of elements for the sphere (cg_col).
struct Geo
{
	double Mk[8][8][8][9];  // stiffness kernel at Gauss point k, [k][a][b][3i+j]: K_e = sum_k eta_k Mk[k] (get_elt_k);
	                        // box: J (dNa/dxj dNb/dxi + delta_ij grad Na . grad Nb); sphere: |J| of the
	                        // strain-rate form 2 (ba1 ba1 + ba2 ba2 + ba3 ba3) + ba4 ba4 + ba5 ba5 + ba6 ba6
	double g[24];           // divergence operator of the element (get_elt_g)
	double gnx[8][8][3];    // dN_a/dx_d at Gauss point k: [k][a][d]; sphere: d/dtheta, d/dphi, d/dr
	double N[8][8];         // N_a at Gauss point k: [k][a]
	double gda[8];          // |J| times the Gauss weight at Gauss point k (E->GDA)
	double tww[8];          // integral of N_a over the element (E->TWW)
	double size[3];         // element sizes (E->ECO.size)
	double area;            // element volume (E->ECO.area)
	double cr[8][8][3];     // [k][a][i]: radial unit vector at Gauss point k . basis vector i of node a (Cc(3, i, a, k));
	                        // box: 1 for i = z, else 0
	double rinv[8];         // 1/r at Gauss point k (box: 1)
	double rsin[8];         // 1/(r sin theta) at Gauss point k (box: 1)
	double wface[4];        // horizontal-average weights of the 4 nodes of the lower face (return_horiz_ave):
	                        // integral of their bilinear shape functions over the face (box: hx hy / 4)
	double gnxc[8][3];      // dN_a/dx_d at the element centre (the pressure point)
	double rinvc, thetac;   // 1/r and theta at the element centre (sphere)
};

// geometry table entries of a level
inline int geo_count(const Lvl &L) { return L.sphere ? L.elx * L.elz : 1; }

// Deterministic reductions: fixed grid, per-block partials, last block sums
// the partials in block order and writes `out[0..nv)`.
struct Red
{
	double *partials;   // RED_MAX_BLOCKS * 8
	unsigned *counter;  // one word, left at 0 after every reduction
};
#define RED_MAX_BLOCKS 304
#define RED_THREADS 256

// fills the geo_count(L) entries of level L (host memory)
void geo_fill_host(const Lvl &L, Geo *g);
void geo_fill_sphere(const Lvl &L, Geo *g);  // geometry.cu

// kernels issued by the launchers below since load (host-side count; a graph
// capture counts its kernels once, each replay is added by the driver)
extern unsigned long long g_kernel_launches;
// launches carry the programmatic-dependent-launch attribute unless 0
extern int g_use_pdl;

// one-time function attributes (large dynamic shared memory); 0 on success
int kernels_init();

// set-up
void launch_assemble(cudaStream_t st, const Lvl &L, const Geo *geo, const double *evi, int aug, double lambda,
                     double *K64, float *K32, double *BI64, float *BI32);
void launch_bpi(cudaStream_t st, const Lvl &L, const Geo *geo, const double *BI64, double *BPI, int precond);

// level operators (T = double or float)
template <typename T> void launch_kmul(cudaStream_t st, const Lvl &L, const T *K, const T *u, T *Au);
template <typename T> void launch_residual(cudaStream_t st, const Lvl &L, const T *K, const T *f, const T *u, T *r);
template <typename T>
void launch_kmul_linesearch(cudaStream_t st, const Lvl &L, const T *K, const T *u, const T *res, T *Au, Red red, double *out2);
template <typename T> void launch_gs_colour(cudaStream_t st, const Lvl &L, const T *K, const T *BI, const T *F, T *d, int colour);
template <typename T>
void launch_gs_small(cudaStream_t st, const Lvl &L, const T *K, const T *BI, const T *F, T *d, int cycles, int zero_start);
// gc: geometry table of the coarse level (TWW)
template <typename T> void launch_project(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, const Geo *gc, const T *AU, T *AD);
// gf: geometry table of the fine level (the sphere's element sizes)
template <typename T> void launch_interp(cudaStream_t st, const Lvl &Lc, const Lvl &Lf, const Geo *gf, const T *AD, T *AU);
template <typename T> void launch_vel_update(cudaStream_t st, int n, T *vel, const T *del, T *res, const T *AU, const double *alpha_num_den, int update_res);
bool gs_small_fits(const Lvl &L, size_t word);
// small FP32 levels: one CTA, vectors in shared memory, padded stencil Kt (63 float4 per node)
bool gs_tiny_fits(const Lvl &L, size_t word);
void launch_tiny_stencil(cudaStream_t st, const Lvl &L, const float *K32, float4 *Kt);
void launch_gs_tiny(cudaStream_t st, const Lvl &L, const float4 *Kt, const float *BI, const float *F, float *d, int cycles,
                    int zero_start);

// The coarse levels of an FP32 multigrid pass as one program run by one
// thread-block cluster (coarse.cu).  Vectors of a level by id:
enum CoVec
{
	CO_VEL,
	CO_DEL,
	CO_RHS,
	CO_RES,
	CO_FL,
	CO_AU,
	CO_NVEC
};
enum CoOpType
{
	CO_GS,      // Gauss-Seidel: vec a relaxed against vec b, `cycles` sweeps, zero start if `zero`
	CO_RESID,   // vec c = vec a - K vec b
	CO_PROJ,    // vec b (level lev-1) = projection of vec a (level lev), stripped
	CO_INTERP,  // vec b (level lev) = interpolation of vec a (level lev-1), stripped
	CO_KDOT,    // vec c = K vec a; alpha = (c . vec b) / (c . c), FP64; if `zero`: then vel += alpha vec a
	CO_UPD,     // vec a += alpha vec b
	CO_DENSE    // `cycles` sweeps of a level as one dense product: vec a = N vec b (zero start, `zero`)
	            // or vec a += N vec b (vec b the residual of vec a; a smoother with a start)
};
#define CO_MAX_LEV 6
#define CO_MAX_OPS 96
#define CO_SMEM_MAX (200 * 1024)
struct CoOp
{
	unsigned char type, lev, a, b, c, zero, local, pad;
	unsigned short cycles;
};
struct CoProg
{
	int n;
	CoOp op[CO_MAX_OPS];
};
struct CoLevels
{
	int nlev;  // levels 0 .. nlev-1
	Lvl L[CO_MAX_LEV];
	const float4 *Kt[CO_MAX_LEV];  // padded stencils
	const float *BI[CO_MAX_LEV];
	float *vec[CO_MAX_LEV][CO_NVEC];
	int win[CO_MAX_LEV];  // ranks on either side of a node's owner that hold its neighbours
	const Geo *geo[CO_MAX_LEV];  // geometry tables (TWW of the projection, sizes of the interpolation)
	double *err;          // set to 1 if a wait of the cluster smoother timed out
	const float *dense[CO_MAX_LEV];  // N (neq x neq, row-major) of a level's smoother, or null
};
// cluster size the device supports for the program (16 or 8); -1 if none
int coarse_init(int *cluster_size);
bool coarse_level_ok(const Lvl &L, int level, int cluster, bool *local);
// the rank window of a level (host): the largest rank distance between a
// node's owner and the owner of one of its neighbours
int coarse_window(const Lvl &L, int cluster);
size_t coarse_smem(const Lvl &L, bool local);
void launch_coarse(cudaStream_t st, const CoLevels &D, const CoProg &P, int cluster, size_t smem);
// The coarsest smoother as a matrix.  With a zero start, `cycles` Gauss-Seidel
// sweeps of level 0 are linear in the right-hand side: d = N f.  Column j of N
// is the smoother (the cluster program's own one-CTA smoother, same colour
// order and arithmetic) applied to the unit vector e_j, one CTA per column.
// work: 2 neq^2 floats; N: neq^2 floats, row-major.
#define CO_DENSE_MAX_EQ 2048
void launch_coarse_dense_build(cudaStream_t st, const Lvl &L, const float4 *Kt, const float *BI, int cycles, float *work, float *N,
                               double *err);
// The same matrix for a level above the one-CTA smoother's size (level 1 of
// the cluster program): column j is `cycles` zero-start colour sweeps against
// e_j, up to 8 columns per CTA with their vectors in shared memory, with the
// level's FP32 stencil K (cg_kidx layout) and 1/diag BI (position order).  A
// smoother with a start d0 is then d = d0 + N (f - K d0), the same N.
// N: neq^2 floats, row-major.
#define CO_DENSE1_MAX_EQ 4096
#define CO_DENSE1_MAX_COLOUR 1024   // nodes of the largest colour
void launch_dense_build_gs(cudaStream_t st, const Lvl &L, const float *K, const float *BI, int cycles, float *N);

// Stencil kernels of the tiled (large) levels, tile.cu: persistent CTAs
// streaming tiles through shared memory with bulk copies
// Element kernels as (hi, lo) FP32 pairs for the double-float assembly
// (assemble.cu): Mk of Geo, and lambda g_a,i g_b,j of the augmented term (zero
// without it).  On the device the table of a level is stored word-major over
// its geometry columns: word w of column c at [w * ncol + c] (GEODF_WORDS
// words per column, in the order of this struct).  The box has one column, so
// its table is this struct; in the spherical segment neighbouring lanes of a
// warp read neighbouring columns.
struct GeoDF
{
	float mh[8][8][8][9], ml[8][8][8][9];
	float lgh[8][8][9], lgl[8][8][9];
};
constexpr int GEODF_WORDS = (int)(sizeof(GeoDF) / sizeof(float));
void geo_df_fill(const Geo &g, int aug, double lambda, GeoDF *out);
// construct_node_ks of a level in double-float arithmetic: splits evi into
// eta2 (8 nel float2), then K64 / K32 / K32lo (the FP32 remainder entry - K32;
// any may be null) and BI64 / BI32.  G: the word-major table of the level's
// geo_count(L) columns
void launch_assemble_df(cudaStream_t st, const Lvl &L, const float *G, const double *evi, float2 *eta2, int aug,
                        double *K64, float *K32, float *K32lo, double *BI64, float *BI32);

// matrix-free FP32 Gauss-Seidel colour of a box level (mf.cu): eta = the
// level's Gauss-point viscosity in FP32 (8 per element), BI = 1/diag K in
// colour-position order
void launch_mf_eta32(cudaStream_t st, const Lvl &L, const double *evi, float *eta);
void launch_mf_gs(cudaStream_t st, const Lvl &L, const float *eta, int aug, double lambda, const float *BI, const float *F,
                  float *d, int colour);

// The finest level's FP64 operator as two FP32 stencils K = Kh + Kl (tile
// layout), applied in double-float arithmetic (tile.cu): out = K u (f null)
// or out = f - K u; FP64 vectors; uv (neq float2) receives u as FP32 pairs
void launch_tile_split(cudaStream_t st, const Lvl &L, const float *Kh, const float *Kl, const double *f, const double *u,
                       float2 *uv, double *out);

int tile_init();                                   // attributes and grid sizes; 0 on success
int tile_error_async(double *host, cudaStream_t st);  // 1 in *host if a stage wait timed out since the last reset
int tile_error_reset_async(cudaStream_t st);         // the tile kernels' error word to zero
int tile_hold_next_copy();                           // failure-path test hook (tile.cu: g_tile_hold)
template <typename T> void launch_tile_gs(cudaStream_t st, const Lvl &L, const T *K, const T *BI, const T *F, T *d, int colour);
template <typename T> void launch_tile_kmul(cudaStream_t st, const Lvl &L, const T *K, const T *u, T *out);
template <typename T> void launch_tile_residual(cudaStream_t st, const Lvl &L, const T *K, const T *f, const T *u, T *out);

// FP64 element operators
void launch_div(cudaStream_t st, const Lvl &L, const Geo *geo, const double *U, double *divU);
void launch_grad(cudaStream_t st, const Lvl &L, const Geo *geo, const double *P, double *gradP);
void launch_strip(cudaStream_t st, const Lvl &L, double *r);

// vectors and reductions
void launch_dot(cudaStream_t st, int n, const double *a, const double *b, Red red, double *out);
void launch_dots4(cudaStream_t st, int n, const double *a0, const double *b0, const double *a1, const double *b1,
                  const double *a2, const double *b2, const double *a3, const double *b3, Red red, double *out);
void launch_axpby(cudaStream_t st, int n, double *y, double a, const double *x, double b);  // y = a*y + b*x
void launch_mul(cudaStream_t st, int n, double *z, const double *a, const double *b);       // z = a*b
// one Uzawa iteration's vector work with device-resident scalars sc[0..4]
void launch_uzawa_precond(cudaStream_t st, int n, const double *BPI, const double *r1, double *z1, Red red, double *sc);
void launch_uzawa_search(cudaStream_t st, int n, double *s2, const double *z1, const double *s1, double *sc, int first);
void launch_uzawa_update(cudaStream_t st, int npno, int neq, double *r2, const double *r1, const double *Ah, double *P,
                         const double *s2, double *V, const double *u1, double *sc, int valid);
void launch_lin2(cudaStream_t st, int n, double *z, double a, const double *x, double b, const double *y);  // z = a*x + b*y
void launch_sub3(cudaStream_t st, int n, double *z, const double *f, const double *a, const double *b);     // z = f - a - b
void launch_copy_d2f(cudaStream_t st, int n, float *dst, const double *src);
void launch_add_f2d(cudaStream_t st, int n, double *dst, const float *src);
void launch_residual64(cudaStream_t st, const Lvl &L, const double *K, const double *f, const double *u, double *r, Red red, double *out_rr);

// viscosity, forces, energy equation, observables (fine level, FP64)
struct Rheo
{
	int tdepv, num_mat;
	double visc0[8], viscE[8], viscT[8], z_layer[8];
	int vmin_on, vmax_on;
	double vmin, vmax;
	int sdepv, sdepv_rheology;      // with sdepv the VMIN/VMAX clamps follow visc_from_S
	double sdepv_expt[8], sdepv_trns[8];
};
void launch_visc_from_T(cudaStream_t st, const Lvl &L, const Geo *geo, const Rheo &r, const double *T, double *evi);
// strain_rate_2_inv (Viscosity_structures.c:979-1086), SQRT form, at the element centres
void launch_strain_rate(cudaStream_t st, const Lvl &L, const Geo *geo, const double *V, double *edot);
// visc_from_S, rheology 1 or 2 (Viscosity_structures.c:744-846), then VMAX/VMIN; edot null: 1 everywhere
void launch_visc_from_S(cudaStream_t st, const Lvl &L, const Geo *geo, const Rheo &r, const double *T, const double *edot,
                        double *evi);
void launch_project_viscosity(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, const Geo *geof, const Geo *geoc,
                              const double *evi_f, double *evi_c, double *work_f, double *work_c);
void launch_buoyancy(cudaStream_t st, const Lvl &L, const Geo *geo, double Ra, const double *T, double *buoy);
// H[z] = horizontal average of T on node layer z (return_horiz_ave)
void launch_horiz_ave(cudaStream_t st, const Lvl &L, const Geo *geo, const double *T, double *H);
void launch_forces(cudaStream_t st, const Lvl &L, const Geo *geo, const double *buoy, double *F);
void launch_v_from_vector(cudaStream_t st, const Lvl &L, const double *U, double *V);
void launch_pg_residual(cudaStream_t st, const Lvl &L, const Geo *geo, const double *T, const double *Tdot, const double *V,
                        double Q0, double *Eres);
void launch_pg_gather(cudaStream_t st, const Lvl &L, const Geo *geo, const double *Eres, double *DTdot);
void launch_predictor(cudaStream_t st, const Lvl &L, double *T, double *Tdot, double dt, double gamma);
void launch_corrector(cudaStream_t st, const Lvl &L, double *T, double *Tdot, const double *DTdot, double dt, double gamma);
void launch_tmax(cudaStream_t st, int n, const double *T, Red red, double *out);
void launch_adv_timestep(cudaStream_t st, const Lvl &L, const Geo *geo, const double *V, Red red, double *out_min_step);
void launch_conform_T(cudaStream_t st, const Lvl &L, double *T);
void launch_heat_flux(cudaStream_t st, const Lvl &L, const Geo *geo, const double *T, const double *V, double *hf_work,
                      Red red, double *out_nut_nub);
void launch_vrms(cudaStream_t st, const Lvl &L, const Geo *geo, const double *V, Red red, double *out);
// The fields of an output step (heat_flux, Process_buoyancy.c:63-203, and
// averages, Process_velocity.c:179-224) from the resident T, V and viscosity:
// f (3 nno): heatflux with the surface nodes replaced, heatflux_adv, flux;
// H (6 noz): layer means T, vrms, Vi, Rho, F, f; surf (2 nsf): shflux, bhflux;
// scal (3): Nut, Nub, Vrms.  scratch: nno, ue: 3 nel, sums: 6 words.
void launch_output_fields(cudaStream_t st, const Lvl &L, const Geo *geo, const double *T, const double *V, const double *evi, Red red,
                          double *f, double *scratch, double *ue, double *H, double *surf, double *sums, double *scal);
