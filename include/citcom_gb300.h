/*
 * citcom_gb300 — GB300 (sm_103a) implementation of CitcomCU's per-timestep
 * hot path behind a plain C ABI.
 *
 * The entry points mirror the reference routines that the CitcomCU driver
 * calls (Drive_solvers.c:45-165, Citcom.c:111-161); each one names the
 * routine it replaces.  Arguments are plain pointers and sizes in the
 * reference's own layouts, all 0-based:
 *   node     n = z + x*noz + y*noz*nox   (Construct_arrays.c:78-81, minus 1)
 *   velocity U[3n+d], d = 0 x, 1 y, 2 z (E->U, Construct_arrays.c:158-165)
 *   pressure P[e], e = ez + ex*elz + ey*elz*elx (E->P + 1)
 *   nodal    T[n], Tdot[n] (E->T + 1, E->Tdot + 1)
 *   V        V[d*nno + n] (E->V[d+1] + 1 for d = 0, 1, 2)
 *   EVI      evi[8e + k], Gauss point k (E->EVI[lev] + 1)
 * Host pointers are copied to and from the device inside the call; the
 * *_device variants take device pointers and do no host traffic.
 *
 * Every function returns CITCOM_GPU_OK (0) or a negative error code; the
 * message is available from citcom_gpu_error_string() (with a null handle:
 * the reason the last citcom_gpu_create of the process failed).  Setting the
 * environment variable CITCOM_GPU_VERBOSE=1 prints one line per Uzawa
 * iteration in the spirit of the reference's generate_log_message;
 * CITCOM_GPU_NO_GRAPH=1 launches the multigrid pass kernel by kernel instead
 * of replaying it as a CUDA graph (for kernel profilers); CITCOM_GPU_NO_PDL=1
 * launches without programmatic dependent launch; CITCOM_GPU_LEVEL_TIMING=1
 * times every smoother call per level (no graph) and prints the totals when
 * the handle is destroyed.  There is no CPU
 * fallback: without a usable CUDA device citcom_gpu_create fails.
 *
 * Scope: the Cartesian box with uniform spacing per axis on every multigrid
 * level, or the regional spherical shell segment (Geometry=Rsphere);
 * free-slip walls (the reference's default reflecting sides), T fixed at the
 * top (0) and bottom (1), insulating sides, one device.
 */
#ifndef CITCOM_GB300_H
#define CITCOM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define CITCOM_GPU_OK 0
#define CITCOM_GPU_ERR_ARG -1
#define CITCOM_GPU_ERR_CUDA -2
#define CITCOM_GPU_ERR_STATE -3
#define CITCOM_GPU_ERR_NOCONV -4

#define CITCOM_GPU_FP64 0   /* plain: multigrid, smoothing and transfers in FP64 */
#define CITCOM_GPU_MIXED 1  /* FP32 multigrid inside FP64 iterative refinement */

typedef struct citcom_gpu citcom_gpu;

/* Problem and solver controls; field names follow E->control / E->mesh /
 * E->viscosity of the reference (Instructions.c:690-1060). */
typedef struct citcom_gpu_config
{
	int levels;          /* mesh.levels: levmin = 0 .. levmax = levels-1 */
	int mgunit[3];       /* mgunitx, mgunity, mgunitz */
	double dimen[3];     /* dimenx, dimeny, dimenz */
	double rayleigh;     /* control.Atemp */
	double Q0;           /* rad_heat.total */
	/* rheology: tdepv 0 -> eta = visc0[mat]; 1 -> rheol 3 */
	int tdepv, num_mat;
	double visc0[8], viscE[8], viscT[8], z_layer[8];
	int vmin_on, vmax_on;
	double vmin, vmax;
	/* Stokes solver */
	int aug_lagr;
	double aug_number;
	int precond;
	int mg_cycle, down_heavy, up_heavy, vlowstep, vhighstep, piterations;
	double accuracy;
	/* energy equation */
	int adv_sub_iterations;
	double finetunedt, fixed_timestep;
	/* CITCOM_GPU_FP64 or CITCOM_GPU_MIXED */
	int precision;
	/* Geometry=Rsphere (control.Rsphere): a regional spherical shell segment
	 * with x, y, z = theta, phi, r; theta_north/south and fi_west/east in
	 * degrees, radius_inner/outer (sphere.ti, to, fi, fo, ri, ro); dimen is
	 * then unused.  0: the Cartesian box (Geometry=cart3d). */
	int sphere;
	double theta[2], fi[2], radius[2];
	/* stress-dependent viscosity (viscosity.SDEPV, Viscosity_structures.c:
	 * 155-162, 286-307): rheology 1 or 2 of visc_from_S, power-law exponent
	 * and transition strain rate per material, the outer iteration's misfit,
	 * iteration cap and damping of general_stokes_solver (Drive_solvers.c:45-165) */
	int sdepv, sdepv_rheology;
	double sdepv_expt[8], sdepv_trns[8];
	double sdepv_misfit, sdepv_iter_damp;
	int max_sdep_visc_iter;
	/* Uzawa stopping rule.  CITCOM_GPU_STOP_REFERENCE (0): the reference's,
	 * dv/v and dp/p below accuracy or piterations iterations
	 * (Stokes_flow_Incomp.c:393, 442-443).  CITCOM_GPU_STOP_RESIDUAL (1): no
	 * counterpart in the reference; the solve runs until both FP64 residuals
	 * of the solution are at most accuracy: |F - K U - G P| / |F| (momentum)
	 * and |B U| / (|U| sqrt(npno/neq)) (continuity), or piterations Uzawa
	 * iterations (see citcom_gpu_solve_Ahat_p_fhat). */
	int stop_rule;
} citcom_gpu_config;

#define CITCOM_GPU_STOP_REFERENCE 0
#define CITCOM_GPU_STOP_RESIDUAL 1

/* Time-step bookkeeping that PG_timestep updates in E->advection / E->monitor. */
typedef struct citcom_gpu_advection
{
	double timestep;            /* advection.timestep (out) */
	double elapsed_time;        /* monitor.elapsed_time (in/out) */
	double T_interior;          /* monitor.T_interior (out) */
	int last_sub_iterations;    /* advection.last_sub_iterations (out) */
} citcom_gpu_advection;

/* Counters of the last Stokes solve. */
typedef struct citcom_gpu_stats
{
	int uzawa_iterations;       /* *steps_max of solve_Ahat_p_fhat */
	int del2_calls;             /* solve_del2_u calls */
	int mg_passes;              /* multi_grid calls */
	double initial_residual;    /* return value of solve_Ahat_p_fhat */
	double stokes_ms;           /* device time of the last solve (CUDA events) */
	double energy_ms;           /* device time of the last PG_timestep of step_resident */
	double smoother_ms;         /* device time of the finest-level Gauss-Seidel calls */
	int smoother_sweeps;        /* finest-level sweeps (8 colour launches each) in smoother_ms */
	unsigned long long kernel_launches;  /* kernels launched by the library since it was loaded */
	int visc_iterations;        /* viscosity iterations of general_stokes_solver (1 unless SDEPV) */
	double visc_misfit;         /* |dU| / |U| of the last stress-dependent iteration */
	int warm_start;             /* 1: the attached network's guess started the Uzawa solve */
	double warm_residual;       /* the Uzawa initial residual |B V| / sqrt(npno) after the head, from the network's guess */
	double base_residual;       /* the same of the resident U, P it was compared with */
	double pass_ms;             /* device time of the multigrid passes (multi_grid calls) */
	/* residual rule only (CITCOM_GPU_STOP_RESIDUAL): the FP64 residuals at the
	 * end of the last Uzawa solve and the velocity corrections it made */
	double final_momentum;      /* |F - K U - G P| / |F| */
	double final_continuity;    /* |B U| / (|U| sqrt(npno/neq)) */
	int corrections;
	int warm_compared;          /* 1: both starts' heads ran (base_residual is then set) */
	double assembly_ms;         /* device time of the last operator assembly inside stokes_resident */
} citcom_gpu_stats;

/* Allocates every device buffer the solver will use (on the current
 * device) and precomputes the mesh geometry.  Replaces the reference's
 * set-up of the solver arrays (Instructions.c:166-398, construct_* in
 * Construct_arrays.c). */
int citcom_gpu_create(const citcom_gpu_config *cfg, citcom_gpu **out);
void citcom_gpu_destroy(citcom_gpu *h);
const char *citcom_gpu_error_string(const citcom_gpu *h);
/* dims = {nox, noy, noz, nno, nel, neq} of level lev */
int citcom_gpu_level_dims(const citcom_gpu *h, int lev, int dims[6]);

/* get_system_viscosity (Viscosity_structures.c:369) from nodal T, followed by
 * project_viscosity (Solver_multigrid.c:398) to every coarser level. */
int citcom_gpu_get_system_viscosity(citcom_gpu *h, const double *T);
/* Use the caller's viscosity at the Gauss points of level lev (E->EVI[lev]+1). */
int citcom_gpu_set_viscosity(citcom_gpu *h, int lev, const double *evi);
int citcom_gpu_get_viscosity(citcom_gpu *h, int lev, double *evi);
/* construct_stiffness_B_matrix (Construct_arrays.c:834): assembles the node
 * stencils, 1/diag(K) on every level and the pressure preconditioner BPI. */
int citcom_gpu_construct_stiffness_B_matrix(citcom_gpu *h);
/* thermal_buoyancy (Pan_problem_misc_functions.c:83) + assemble_forces
 * (Element_calculations.c:74): F (neq) from T (nno); buoyancy optional (nno). */
int citcom_gpu_assemble_forces(citcom_gpu *h, const double *T, double *F, double *buoyancy);

/* solve_Ahat_p_fhat (Stokes_flow_Incomp.c:295): Uzawa / Schur-complement
 * PCG with the multigrid velocity solve.  V (neq) and P (npno) are updated
 * in place; *steps_max is the iteration cap on entry and the iteration
 * count on return; *initial_residual receives the reference's return value.
 * With stop_rule CITCOM_GPU_STOP_RESIDUAL the loop tests the continuity
 * residual (from the recursively updated B V) before every iteration; once
 * it is at most imp, the momentum residual is evaluated with the FP64
 * operator, and if it is above imp a velocity correction
 * V += K^-1 (F - G P - K V) (the reference's own head, :360-366, solved to
 * imp/2 relative to |F|) follows, B V is recomputed and the iteration
 * restarts its search direction if continuity is above imp again.  At most 8
 * corrections are made per solve. */
int citcom_gpu_solve_Ahat_p_fhat(citcom_gpu *h, double *V, double *P, const double *F, double imp, int *steps_max,
                                 double *initial_residual);
int citcom_gpu_solve_Ahat_p_fhat_device(citcom_gpu *h, double *dV, double *dP, const double *dF, double imp, int *steps_max,
                                        double *initial_residual);
/* solve_constrained_flow_iterative (Stokes_flow_Incomp.c:50) with
 * v_from_vector: U, P updated in place with control.accuracy and
 * control.p_iterations; nodal V (3*nno) written. */
int citcom_gpu_solve_constrained_flow_iterative(citcom_gpu *h, double *U, double *P, const double *F, double *V);

/* general_stokes_solver (Drive_solvers.c:45) for a Newtonian rheology:
 * forces from T, viscosity from T when tdepv, stiffness, Uzawa, V.
 * U, P are in/out (warm start), V (3*nno) out. */
int citcom_gpu_general_stokes_solver(citcom_gpu *h, const double *T, double *U, double *P, double *V);

/* PG_timestep (Advection_diffusion.c:251): T, Tdot (nno) in/out, V (3*nno) in. */
int citcom_gpu_PG_timestep(citcom_gpu *h, double *T, double *Tdot, const double *V, citcom_gpu_advection *adv);

/* heat_flux (Process_buoyancy.c:63): surface Nusselt numbers; and the
 * volume-rms velocity sqrt(int |u|^2 dV / V). */
int citcom_gpu_heat_flux(citcom_gpu *h, const double *T, const double *V, double *nut, double *nub);
int citcom_gpu_vrms(citcom_gpu *h, const double *V, double *vrms);

/* Whole time step on device-resident state (T, Tdot, U, P, V held by the
 * handle): PG_timestep then general_stokes_solver, the order of the
 * reference's time loop (Citcom.c:111-161).  Load/store move the state. */
int citcom_gpu_load_state(citcom_gpu *h, const double *T, const double *Tdot, const double *U, const double *P);
int citcom_gpu_store_state(citcom_gpu *h, double *T, double *Tdot, double *U, double *P, double *V);
int citcom_gpu_stokes_resident(citcom_gpu *h);
int citcom_gpu_step_resident(citcom_gpu *h, citcom_gpu_advection *adv);
int citcom_gpu_last_stats(const citcom_gpu *h, citcom_gpu_stats *s);
/* Output step.  The reference computes the fields of an output step on the
 * host (heat_flux, Process_buoyancy.c:63-203; averages,
 * Process_velocity.c:179-224) and writes them as ASCII (output_velo_related,
 * Output.c:54-170).  citcom_gpu_output_async computes them on the device from
 * the resident state (T, V, P, viscosity), copies them into device staging on
 * the handle's stream, and from there to the caller's host buffers on a second
 * stream, so that the copy to the host overlaps the work queued after it (the
 * next time step).  Host buffers should be pinned for the overlap; any pointer
 * may be null.  They are complete once citcom_gpu_output_wait returns; a
 * second call first waits for the previous one's copies.  The staging
 * (8 nno + 4 nel doubles) is allocated on the first call.  Composition
 * (Have.C), the adiabat (Have.Tadi) and topography (slice.tpg) are not
 * computed. */
typedef struct
{
	double *T;            /* nno */
	double *V;            /* 3 x nno (V[1], V[2], V[3]) */
	double *P;            /* nel */
	double *heatflux;     /* nno: E->heatflux as heat_flux leaves it (u_z |T - <T>|) */
	double *heatflux_adv; /* nno: E->heatflux_adv (u_z (T - <T>)) */
	double *Have;         /* 6 x noz: Have.T, vrms, Vi, Rho, F, f (.ave columns 1-6) */
	double *surf;         /* 2 x nox noy: slice.shflux, slice.bhflux */
	double *scalars;      /* 3: slice.Nut, slice.Nub, Vrms */
} citcom_gpu_output;
int citcom_gpu_output_async(citcom_gpu *h, const citcom_gpu_output *out);
int citcom_gpu_output_wait(citcom_gpu *h);
/* Residuals of the resident solution, in FP64: out[0] = |F - K U - G P| / |F|
 * (momentum), out[1] = |div U| / (|U| sqrt(npno/neq)) (continuity).  No
 * counterpart in the reference, which stops on the relative increments
 * dv/v and dp/p (Stokes_flow_Incomp.c:393, 442-443). */
int citcom_gpu_stokes_residuals(citcom_gpu *h, double out[2]);

/* Failure-path test hook (no counterpart in the reference).  The stencil
 * kernels of the large levels wait, with a limit of about a second, for the
 * bulk copies of their stencil tiles; when a wait runs out the kernel sets an
 * error word, issues no further copy, waits for the copies it has in flight
 * and returns, and the calling entry point returns CITCOM_GPU_ERR_CUDA with
 * the reason (the word is then cleared; the context stays usable).  After this
 * call the next such kernel to start arms one stage without issuing its copy,
 * so that exactly one wait runs out.  For tests of that path only. */
int citcom_gpu_test_hold_tile_copy(void);

/* Single operators of level lev, host buffers (the kernels the solver uses;
 * exposed for parity checks against the reference's routines). */
/* n_assemble_del2_u (Element_calculations.c:552), stripped */
int citcom_gpu_op_kmul(citcom_gpu *h, int lev, const double *u, double *Au);
/* gauss_seidel (General_matrix_functions.c:1160), 8-colour order; d0 in/out
 * when guess != 0; Ad = K d0 on return.  In the mixed configuration it runs
 * the FP32 smoother of a level below the finest (values rounded to float). */
int citcom_gpu_op_gauss_seidel(citcom_gpu *h, int lev, double *d0, const double *F, double *Ad, int cycles, int guess);
/* project_vector (Solver_multigrid.c:72) fine_lev -> fine_lev-1, stripped */
int citcom_gpu_op_project(citcom_gpu *h, int fine_lev, const double *AU, double *AD);
/* interp_vector (Solver_multigrid.c:173) coarse_lev -> coarse_lev+1, stripped */
int citcom_gpu_op_interp(citcom_gpu *h, int coarse_lev, const double *AD, double *AU);
/* assemble_div_u / assemble_grad_p (Element_calculations.c:691, 727) */
int citcom_gpu_op_div(citcom_gpu *h, int lev, const double *U, double *divU);
int citcom_gpu_op_grad(citcom_gpu *h, int lev, const double *P, double *gradP);
/* multi_grid (General_matrix_functions.c:525): d1 out, F in/out (residual);
 * in the mixed configuration one FP32 pass on F rounded to float */
int citcom_gpu_op_multi_grid(citcom_gpu *h, double *d1, double *F, double *residual);
/* solve_del2_u (General_matrix_functions.c:368) on the finest level */
int citcom_gpu_op_solve_del2_u(citcom_gpu *h, double *d0, const double *F, double acc, int *valid);
/* BI (neq, 1/diag K) and BPI (nel) of level lev as the solver holds them */
int citcom_gpu_op_diagonals(citcom_gpu *h, int lev, double *BI, double *BPI);

/* Surface Nusselt numbers of heat_flux (Process_buoyancy.c:63) for callers
 * that cannot allocate device memory.  No counterpart in the reference.
 * Everything it needs beyond its inputs and outputs lives in one fixed device
 * array inside the library (about 4.4 MB, held by every GPU that loads the
 * library until the process exits); it calls no cudaMalloc/cudaFree and needs
 * no handle.  dT (nno) and dV (3*nno, layout of V above) are DEVICE pointers
 * of a nox*noy*noz Cartesian box of size dimen (box geometry only: it takes
 * no spherical segment, whose Nusselt numbers come from citcom_gpu_heat_flux);
 * nut/nub receive the results on the host.  Meshes above
 * CITCOM_GPU_NOALLOC_MAX_NODES nodes or CITCOM_GPU_NOALLOC_MAX_ELEMENTS
 * elements are rejected with CITCOM_GPU_ERR_ARG and a message on stderr.
 * Runs on the legacy default stream and returns after the result is on the
 * host.  That stream does not wait for work on non-blocking streams, so dT
 * and dV must be complete before the call: synchronise the stream that
 * writes them first.  The first call on a
 * device looks up the array's device address (once per device, with that
 * device current), so make the first call before any stream capture.  All
 * calls share the one array: calls that overlap on the GPU race and must be
 * serialised by the caller. */
#define CITCOM_GPU_NOALLOC_MAX_NODES 274625
#define CITCOM_GPU_NOALLOC_MAX_ELEMENTS 262144
int citcom_gpu_heat_flux_noalloc(int nox, int noy, int noz, const double dimen[3], const double *dT, const double *dV,
                                 double *nut, double *nub);

/* Learned warm start of the Stokes solve.  No counterpart in the reference,
 * which starts solve_Ahat_p_fhat (Stokes_flow_Incomp.c:295) from the previous
 * time step's U and P.  A 3D convolutional encoder-decoder on the node grid of
 * multigrid level `level` (-1: the second finest) maps T and log10 of the
 * viscosity to velocity and pressure; BF16 weights and activations, FP32
 * accumulation on the tensor cores, FP32 master weights trained with Adam on
 * snapshots of converged solves of the same handle.  When attached, every
 * Uzawa solve of the handle (solve_Ahat_p_fhat and everything that calls it)
 * runs its head -- the velocity correction for the given pressure and the
 * initial residual |div V| / sqrt(npno) that solve_Ahat_p_fhat returns -- for
 * the network's guess as well as for the resident U, P (the previous solution,
 * or zero), and iterates from the pair with the smaller initial residual (see
 * citcom_nn_set_check_interval for comparing less often).  The solve then runs
 * to the same stopping rule, so the network changes only the iteration count
 * (at the price of one extra velocity solve per comparison).  The network
 * must be destroyed before its solver handle, or at least not used after it. */
typedef struct citcom_nn citcom_nn;
int citcom_nn_create(citcom_gpu *h, int level, unsigned seed, int capacity, citcom_nn **out);
void citcom_nn_destroy(citcom_nn *n);
const char *citcom_nn_error_string(const citcom_nn *n);
/* info: nox, noy, noz of the network grid, parameter count, recorded snapshots, level */
int citcom_nn_info(const citcom_nn *n, int info[6]);
/* parameters, FP32, per layer W[cout][cin][27] (tap 9(dy+1)+3(dx+1)+(dz+1)) then b[cout] */
int citcom_nn_get_params(citcom_nn *n, float *w);
int citcom_nn_set_params(citcom_nn *n, const float *w);
/* output scales: velocity and pressure per unit RMS of the temperature anomaly
 * (T minus its horizontal mean), and a pressure offset; set by the first record */
int citcom_nn_get_scales(const citcom_nn *n, double s[3]);
int citcom_nn_set_scales(citcom_nn *n, const double s[3]);
/* adds the handle's resident (T, viscosity, U, P) to the training set (a ring of `capacity`) */
int citcom_nn_record(citcom_nn *n);
/* `steps` Adam steps on random minibatches of `batch` snapshots; loss of the last step */
int citcom_nn_train(citcom_nn *n, int steps, int batch, double lr, double *loss);
/* What the network predicts (set before the first record).
 * CITCOM_NN_ABSOLUTE: U and P from T and the viscosity, as above.
 * CITCOM_NN_INCREMENT: the change of U and P since the handle's last Stokes
 * solve, from the change of T since that solve (T - T_sol, restricted to the
 * network grid, minus its horizontal mean, over its RMS) and the viscosity.
 * Training samples are the differences between consecutive records of one
 * state sequence (a load_state starts a new sequence; its first record
 * only remembers the state).  An attached network then offers (U + dU,
 * P + dP) as the guess of each Uzawa solve that follows a completed solve of
 * the same sequence, compared with the previous step's (U, P) as in the
 * absolute mode. */
#define CITCOM_NN_ABSOLUTE 0
#define CITCOM_NN_INCREMENT 1
int citcom_nn_set_mode(citcom_nn *n, int mode);
/* How often the network's start is compared with the resident one (both
 * heads run and the start with the smaller initial residual is kept).
 * every = 1 (the default): every solve.  every = k > 1: every k-th solve the
 * network could start, and also whenever its start's initial residual
 * exceeds 4x that of the last comparison it won; between comparisons the
 * last winner starts alone (no second head).  Resets the comparison
 * history. */
int citcom_nn_set_check_interval(citcom_nn *n, int every);
/* on != 0: warm-start every Stokes solve of the handle */
int citcom_nn_attach(citcom_nn *n, int on);
/* the guess for the resident T and viscosity: U (neq), P (nel) on the host
 * (absolute mode only) */
int citcom_nn_predict(citcom_nn *n, double *U, double *P);
/* checks of the network alone, host buffers in the network's scaled units:
 * x (V x 2: temperature anomaly / its RMS, (log10 eta + 1.5) / 1.5), y and t
 * (V x 4: u, v, w, p in units of the scales above times the anomaly RMS);
 * loss = mean over V x 4 of (y - t)^2 and its gradient in the parameter layout */
int citcom_nn_forward(citcom_nn *n, const float *x, float *y);
int citcom_nn_loss_grad(citcom_nn *n, const float *x, const float *t, double *loss, float *grad);

#ifdef __cplusplus
}
#endif
#endif
