/*
 * CPU restatement of CitcomCU's per-timestep hot path (Stokes solve and SUPG
 * energy step) for a Cartesian box with a uniform grid per axis.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against; the product never links or calls it.  It is itself pinned against
 * the unchanged reference (oracle/ref, built into oracle/_ref) through the
 * golden fixtures under tests/golden.
 *
 * Everything is computed in FP64 and follows the reference step by step; each
 * function names the reference routine (file:line) it restates.  Arrays are
 * 0-based: node n = z + x*noz + y*noz*nox, equation 3n+d, element/pressure
 * e = ez + ex*elz + ey*elz*elx.
 */
#ifndef CITCOM_ORACLE_H
#define CITCOM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORACLE_MAX_LEVELS 12
#define ORACLE_MAX_MAT 8

typedef struct oracle_params
{
	int levels;            /* levmin = 0 .. levmax = levels-1 */
	int mgunit[3];         /* coarsest elements along x, y, z */
	double dimen[3];       /* box size along x, y, z */
	double rayleigh;
	double Q0;
	int tdepv;             /* 0: eta = visc0[mat]; 1: rheol 3 */
	int num_mat;
	double visc0[ORACLE_MAX_MAT], viscE[ORACLE_MAX_MAT], viscT[ORACLE_MAX_MAT];
	double z_layer[ORACLE_MAX_MAT];
	int vmin_on, vmax_on;
	double vmin, vmax;
	int aug_lagr;
	double aug_number;
	int precond;
	int mg_cycle, down_heavy, up_heavy, vlowstep, vhighstep, piterations;
	double accuracy;
	int adv_sub_iterations;
	double finetunedt, fixed_timestep;
	int gs_colored;        /* 0: lexicographic (reference order); 1: 8-colour */
	/* stress-dependent viscosity (SDEPV, Viscosity_structures.c:744-846) and
	   the viscosity iteration of general_stokes_solver (Drive_solvers.c:120-159) */
	int sdepv, sdepv_rheology;
	double sdepv_expt[ORACLE_MAX_MAT], sdepv_trns[ORACLE_MAX_MAT];
	double sdepv_misfit, sdepv_iter_damp;
	int max_sdep_visc_iter;
	/* 0: the reference's Uzawa stopping rule (dv/v, dp/p); 1: the residual
	   rule of the GPU library (both FP64 residuals at most accuracy, velocity
	   corrections), restated in oracle_solve_Ahat_p_fhat */
	int stop_rule;
} oracle_params;

typedef struct oracle oracle;

oracle *oracle_create(const oracle_params *p);
void oracle_destroy(oracle *o);

/* sizes of a level: nox, noy, noz, nno, nel, neq */
void oracle_level_dims(const oracle *o, int lev, int dims[6]);

/* state access (fine level) */
double *oracle_T(oracle *o);
double *oracle_Tdot(oracle *o);
double *oracle_U(oracle *o);      /* neq */
double *oracle_P(oracle *o);      /* npno */
double *oracle_F(oracle *o);      /* neq */
double *oracle_V(oracle *o, int d);   /* nno, d = 0,1,2 */
double *oracle_buoyancy(oracle *o);
double *oracle_EVI(oracle *o, int lev);   /* 8 per element */
double *oracle_BI(oracle *o, int lev);
double *oracle_BPI(oracle *o, int lev);
unsigned *oracle_vflags(oracle *o, int lev);   /* bit0 x, bit1 y, bit2 z constrained */
double *oracle_stencil(oracle *o, int lev);    /* 243 per node: [27 neighbours][3x3] */
double oracle_timestep(const oracle *o);
double oracle_elapsed_time(const oracle *o);
double oracle_T_interior(const oracle *o);
void oracle_set_timestep(oracle *o, double dt);

/* set-up steps (each restates the named reference routine) */
void oracle_thermal_buoyancy(oracle *o);
void oracle_assemble_forces(oracle *o);
void oracle_get_system_viscosity(oracle *o);
void oracle_project_viscosity(oracle *o);
void oracle_construct_stiffness(oracle *o);

/* operators on a level */
void oracle_kmul(oracle *o, int lev, const double *u, double *Au, int strip);
void oracle_strip_bcs(oracle *o, int lev, double *r);
void oracle_gauss_seidel(oracle *o, int lev, double *d0, const double *F, double *Ad, int cycles, int guess);
void oracle_project_vector(oracle *o, int fine_lev, const double *AU, double *AD);
void oracle_interp_vector(oracle *o, int coarse_lev, const double *AD, double *AU);
void oracle_div_u(oracle *o, int lev, const double *U, double *divU);
void oracle_grad_p(oracle *o, int lev, const double *P, double *gradP);

/* solvers */
double oracle_multi_grid(oracle *o, double *d1, double *F, double acc);
int oracle_solve_del2_u(oracle *o, double *d0, double *F, double acc, int *mg_calls);
double oracle_solve_Ahat_p_fhat(oracle *o, double *V, double *P, const double *F, double imp, int *steps, int *del2_calls, int *mg_calls);
/* residual rule of the last solve: momentum, continuity, corrections */
void oracle_last_residuals(const oracle *o, double out[3]);
/* general_stokes_solver: conform BCs, forces, viscosity, stiffness, Uzawa, V */
double oracle_stokes(oracle *o, int *steps, int *del2_calls, int *mg_calls);

/* energy equation and observables */
void oracle_pg_timestep(oracle *o);
void oracle_heat_flux(oracle *o, double *nut, double *nub);
double oracle_vrms(oracle *o);

#ifdef __cplusplus
}
#endif
#endif
