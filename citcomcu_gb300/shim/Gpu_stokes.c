/*
 * Gpu_stokes.c -- the reference-side shim that puts CitcomCU's Stokes solve
 * and energy step on the GB300 library (include/citcom_gb300.h).
 *
 * A CitcomCU maintainer adds this file to the reference's src/ (CFILES),
 * compiles it with the same -D flags as the other objects (the struct layout
 * of All_variables depends on them) and links with -lcitcom_gb300.  Two
 * reference files are compiled with renames so that their own versions of
 * the replaced routines step aside:
 *   Stokes_flow_Incomp.c  -Dsolve_constrained_flow_iterative=ref_solve_constrained_flow_iterative
 *                         -Dsolve_Ahat_p_fhat=ref_solve_Ahat_p_fhat
 *   Construct_arrays.c    -Dconstruct_stiffness_B_matrix=ref_construct_stiffness_B_matrix
 * The replaced routines are solve_constrained_flow_iterative and
 * solve_Ahat_p_fhat (Stokes_flow_Incomp.c:50, 295), construct_stiffness_B_matrix
 * (Construct_arrays.c:834) and, through the reference's own function pointer
 * E->next_buoyancy_field (Convection.c:90-93), PG_timestep
 * (Advection_diffusion.c:251).  gpu_output_step serves an output step from the
 * device.  Define CITCOM_GPU_WARM_START to attach the learned warm start.
 *
 * The reference's arrays are 1-based for nodes, elements and pressures; the
 * ABI is 0-based, so the shim passes ptr + 1.  In the stock build E->T, E->V
 * and E->EVI are float; the shim converts them through double staging
 * buffers.
 */

#include <stdlib.h>
#include "element_definitions.h"
#include "global_defs.h"
#include "citcom_gb300.h"

static citcom_gpu *G;
static double *Td, *Tdotd, *Vd;

void gpu_PG_timestep(struct All_variables *E);
#ifdef CITCOM_GPU_WARM_START
static void gpu_warm_start_init(struct All_variables *E);
static void gpu_warm_start_learn(struct All_variables *E);
#endif

static void gpu_check(struct All_variables *E, int rc, const char *where)
{
	if(rc != CITCOM_GPU_OK) {
		fprintf(stderr, "%s: %s\n", where, citcom_gpu_error_string(G));
		parallel_process_termination();           /* the reference's abort path */
	}
}

static void gpu_init(struct All_variables *E)
{
	citcom_gpu_config c = {0};
	int i;
	if(G) return;
	if(E->parallel.nproc != 1) { fprintf(stderr, "GPU path runs one rank\n"); parallel_process_termination(); }
	c.levels = E->mesh.levmax + 1;
	c.mgunit[0] = E->mesh.mgunitx; c.mgunit[1] = E->mesh.mgunity; c.mgunit[2] = E->mesh.mgunitz;
	c.dimen[0] = E->mesh.layer[1]; c.dimen[1] = E->mesh.layer[2]; c.dimen[2] = E->mesh.layer[3];
	c.rayleigh = E->control.Atemp; c.Q0 = E->control.Q0;
	c.tdepv = E->viscosity.TDEPV; c.num_mat = E->viscosity.num_mat;
	for(i = 0; i < c.num_mat; i++) {
		c.visc0[i] = E->viscosity.N0[i]; c.viscE[i] = E->viscosity.E[i];
		c.viscT[i] = E->viscosity.T[i];  c.z_layer[i] = E->viscosity.zbase_layer[i];
	}
	c.vmin_on = E->viscosity.MIN; c.vmin = E->viscosity.min_value;
	c.vmax_on = E->viscosity.MAX; c.vmax = E->viscosity.max_value;
	c.aug_lagr = E->control.augmented_Lagr; c.aug_number = E->control.augmented;
	c.precond = E->control.precondition;
	c.mg_cycle = E->control.mg_cycle; c.down_heavy = E->control.down_heavy; c.up_heavy = E->control.up_heavy;
	c.vlowstep = E->control.v_steps_low; c.vhighstep = E->control.v_steps_high;
	c.piterations = E->control.p_iterations; c.accuracy = E->control.accuracy;
	c.adv_sub_iterations = E->advection.temp_iterations;
	c.finetunedt = E->advection.fine_tune_dt; c.fixed_timestep = E->advection.fixed_timestep;
	c.precision = CITCOM_GPU_MIXED;   /* or CITCOM_GPU_FP64 */
	c.stop_rule = CITCOM_GPU_STOP_REFERENCE;   /* or CITCOM_GPU_STOP_RESIDUAL: both FP64 residuals <= accuracy */
	if(E->control.Rsphere) {          /* regional spherical shell segment */
		c.sphere = 1;
		c.theta[0] = E->sphere.ti; c.theta[1] = E->sphere.to;     /* degrees */
		c.fi[0] = E->sphere.fi;    c.fi[1] = E->sphere.fo;
		c.radius[0] = E->sphere.ri; c.radius[1] = E->sphere.ro;
	}
	gpu_check(E, citcom_gpu_create(&c, &G), "citcom_gpu_create");
#ifdef CITCOM_GPU_WARM_START
	gpu_warm_start_init(E);
#endif
	/* the energy step through the reference's own hook (Convection.c:90-93):
	   the first Stokes solve runs before the time loop, so no reference file
	   needs editing */
	E->next_buoyancy_field = gpu_PG_timestep;
	Td = malloc(sizeof(double) * E->lmesh.nno);
	Tdotd = malloc(sizeof(double) * E->lmesh.nno);
	Vd = malloc(sizeof(double) * 3 * E->lmesh.nno);
}

/* replaces Stokes_flow_Incomp.c:50 */
void solve_constrained_flow_iterative(struct All_variables *E)
{
	int n, d;
	gpu_init(E);
	gpu_check(E, citcom_gpu_solve_constrained_flow_iterative(G, E->U, E->P + 1, E->F, Vd),
	          "solve_constrained_flow_iterative");
	for(d = 1; d <= 3; d++)
		for(n = 1; n <= E->lmesh.nno; n++)
			E->V[d][n] = Vd[(d - 1) * E->lmesh.nno + n - 1];
#ifdef CITCOM_GPU_WARM_START
	gpu_warm_start_learn(E);
#endif
}

/* replaces Stokes_flow_Incomp.c:295 */
float solve_Ahat_p_fhat(struct All_variables *E, double *V, double *P, double *F, double imp, int *steps_max)
{
	double r0 = 0.0;
	gpu_init(E);
	gpu_check(E, citcom_gpu_solve_Ahat_p_fhat(G, V, P + 1, F, imp, steps_max, &r0), "solve_Ahat_p_fhat");
	return (float)r0;
}

/* installed over construct_stiffness_B_matrix: compile Construct_arrays.c with
   -Dconstruct_stiffness_B_matrix=ref_construct_stiffness_B_matrix so the host
   assembly stays off the time step; same rebuild rule as Construct_arrays.c:849 */
void construct_stiffness_B_matrix(struct All_variables *E)
{
	static int been_here = 0;
	int i;
	gpu_init(E);
	if(been_here && !(E->viscosity.update_allowed && E->monitor.solution_cycles % E->control.KERNEL == 0))
		return;
	for(i = 1; i <= E->lmesh.nno; i++) Td[i - 1] = E->T[i];
	gpu_check(E, citcom_gpu_get_system_viscosity(G, Td), "get_system_viscosity");
	gpu_check(E, citcom_gpu_construct_stiffness_B_matrix(G), "construct_stiffness_B_matrix");
	been_here = 1;
}

/* installed through the hook: E->next_buoyancy_field = gpu_PG_timestep */
void gpu_PG_timestep(struct All_variables *E)
{
	citcom_gpu_advection adv;
	int n, d;
	gpu_init(E);
	for(n = 1; n <= E->lmesh.nno; n++) { Td[n - 1] = E->T[n]; Tdotd[n - 1] = E->Tdot[n]; }
	for(d = 1; d <= 3; d++)
		for(n = 1; n <= E->lmesh.nno; n++) Vd[(d - 1) * E->lmesh.nno + n - 1] = E->V[d][n];
	adv.elapsed_time = E->monitor.elapsed_time;
	E->advection.timesteps++;
	gpu_check(E, citcom_gpu_PG_timestep(G, Td, Tdotd, Vd, &adv), "PG_timestep");
	for(n = 1; n <= E->lmesh.nno; n++) { E->T[n] = Td[n - 1]; E->Tdot[n] = Tdotd[n - 1]; }
	E->advection.timestep = adv.timestep;
	E->monitor.elapsed_time = adv.elapsed_time;
	E->monitor.T_interior = adv.T_interior;
	E->advection.last_sub_iterations = adv.last_sub_iterations;
	E->advection.total_timesteps++;
	thermal_buoyancy(E);                       /* E->buoyancy for assemble_forces */
	E->control.keep_going = E->monitor.solution_cycles < E->advection.max_timesteps;
}

/* the remaining symbols of Stokes_flow_Incomp.o (generate_log_message,
   v_from_vector, vector_from_v, initial_vel_residual, solve_Ahat_p_fhat_new)
   come from the unchanged file, compiled with the two renames above */

/* ------------------------------------------------------------ output step */

static double *Ho, *Hs, *Hsc, *Hflux, *Hadv;   /* pinned: cudaHostAlloc'd */

/* replaces process_new_velocity's averages + output_velo_related input */
void gpu_output_step(struct All_variables *E, int file_number)
{
	citcom_gpu_output o = {0};
	int i, nsf = E->lmesh.nsf, noz = E->lmesh.noz;
	o.Have = Ho; o.surf = Hs; o.scalars = Hsc; o.heatflux = Hflux; o.heatflux_adv = Hadv;
	gpu_check(E, citcom_gpu_output_async(G, &o), "output_async");
	/* ... the next time step may be queued here; the copies overlap it ... */
	gpu_check(E, citcom_gpu_output_wait(G), "output_wait");
	for(i = 1; i <= noz; i++) {
		E->Have.T[i] = Ho[i - 1];           E->Have.vrms[i] = Ho[noz + i - 1];
		E->Have.Vi[i] = Ho[2 * noz + i - 1]; E->Have.Rho[i] = Ho[3 * noz + i - 1];
		E->Have.F[i] = Ho[4 * noz + i - 1];  E->Have.f[i] = Ho[5 * noz + i - 1];
	}
	for(i = 1; i <= nsf; i++) { E->slice.shflux[i] = Hs[i - 1]; E->slice.bhflux[i] = Hs[nsf + i - 1]; }
	for(i = 1; i <= E->lmesh.nno; i++) { E->heatflux[i] = Hflux[i - 1]; E->heatflux_adv[i] = Hadv[i - 1]; }
	E->slice.Nut = Hsc[0]; E->slice.Nub = Hsc[1];
	output_velo_related(E, file_number);
}

#ifdef CITCOM_GPU_WARM_START
/* ------------------------------------------------- learned warm start */
static citcom_nn *NN;

static void gpu_warm_start_init(struct All_variables *E)
{
	/* second-finest level, a ring of 2000 snapshots, increment mode: the
	   network predicts the change of U, P over a time step */
	gpu_check(E, citcom_nn_create(G, -1, 0, 2000, &NN), "citcom_nn_create");
	gpu_check(E, citcom_nn_set_mode(NN, CITCOM_NN_INCREMENT), "citcom_nn_set_mode");
	gpu_check(E, citcom_nn_attach(NN, 1), "citcom_nn_attach");
}

static void gpu_warm_start_learn(struct All_variables *E)
{
	/* learn from the solution; train every 10 steps */
	if(citcom_nn_record(NN) == CITCOM_GPU_OK && E->monitor.solution_cycles % 10 == 0)
		citcom_nn_train(NN, 100, 4, 1e-3, NULL);
}
#endif
