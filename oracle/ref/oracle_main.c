/*
 * Driver that runs the UNCHANGED CitcomCU sources (compiled from the
 * reference tree by oracle/ref/Makefile) on a deck and writes the state the
 * GPU library is checked against.  Test infrastructure only.
 *
 * It follows the time loop of Citcom.c:54-175 (main): read_instructions,
 * one general_stokes_solver before the loop, then per step process_heating,
 * the next_buoyancy_field hook (PG_timestep), process_temp_field (Nu) and
 * general_stokes_solver.  Output writers (process_new_velocity and friends)
 * are not called: the state is written in binary instead, because the
 * reference's ASCII output (Output.c:54-170, 4-6 digits) is too coarse for
 * parity checks.
 *
 * Usage: citcom_ref <deck> <T0.bin|-> <nsteps> <out.bin> [probe]
 *   T0.bin  nno doubles overriding the initial temperature (node order of
 *           Construct_arrays.c:78-81); '-' keeps the deck's own IC.
 *   probe   additionally exercise single operators on deterministic test
 *           vectors (n_assemble_del2_u, gauss_seidel, project_vector,
 *           interp_vector, assemble_div_u, assemble_grad_p, multi_grid,
 *           solve_del2_u) and write their outputs.
 *
 * Record format: 32-byte NUL-padded name, int64 count, count doubles.
 */
#include <mpi.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <sys/types.h>

#include "element_definitions.h"
#include "global_defs.h"

extern int Emergency_stop;

double multi_grid(struct All_variables *, double *, double *, double *, double, int);

static FILE *out;

static void rec_d(const char *name, const double *x, long n)
{
	char nm[32];
	int64_t c = n;
	memset(nm, 0, sizeof(nm));
	strncpy(nm, name, 31);
	fwrite(nm, 1, 32, out);
	fwrite(&c, sizeof(c), 1, out);
	fwrite(x, sizeof(double), (size_t)n, out);
}

/* float in the stock build, double in the promoted build */
static void rec_f(const char *name, const float *x, long n)
{
	double *t = (double *)malloc((size_t)(n + 1) * sizeof(double));
	long i;
	for(i = 0; i < n; i++)
		t[i] = (double)x[i];
	rec_d(name, t, n);
	free(t);
}

static void rec_s(const char *name, double v) { rec_d(name, &v, 1); }

static void test_vector(double *u, int n, double a, double b)
{
	int i;
	for(i = 0; i < n; i++)
		u[i] = sin(a * (double)i + b) + 0.25 * cos(0.013 * (double)i * (double)i);
}

static void probe_operators(struct All_variables *E)
{
	char nm[64];
	int lev;
	const int lmax = E->mesh.levmax, lmin = E->mesh.levmin;
	int cycles;

	for(lev = lmin; lev <= lmax; lev++)
	{
		const int neq = E->lmesh.NEQ[lev], nno = E->lmesh.NNO[lev], npno = E->lmesh.NPNO[lev];
		double *u = calloc(neq + 4, sizeof(double));
		double *au = calloc(neq + 4, sizeof(double));
		double *p = calloc(npno + 4, sizeof(double));
		double *flags = calloc(nno + 1, sizeof(double));
		int i;

		for(i = 1; i <= nno; i++)
			flags[i - 1] = (double)E->NODE[lev][i];
		snprintf(nm, sizeof nm, "NODE_%d", lev);
		rec_d(nm, flags, nno);
		snprintf(nm, sizeof nm, "EVI_%d", lev);
		rec_f(nm, E->EVI[lev] + 1, (long)npno * 8);
		snprintf(nm, sizeof nm, "BI_%d", lev);
		rec_d(nm, E->BI[lev], neq);
		snprintf(nm, sizeof nm, "BPI_%d", lev);
		rec_d(nm, E->BPI[lev] + 1, npno);

		test_vector(u, neq, 0.37, 0.11);
		u[neq] = u[neq + 1] = 0.0;
		snprintf(nm, sizeof nm, "u_%d", lev);
		rec_d(nm, u, neq);
		n_assemble_del2_u(E, u, au, lev, 1);
		snprintf(nm, sizeof nm, "Ku_%d", lev);
		rec_d(nm, au, neq);

		assemble_div_u(E, u, p, lev);
		snprintf(nm, sizeof nm, "divu_%d", lev);
		rec_d(nm, p + 1, npno);

		test_vector(p + 1, npno, 0.21, 0.5);
		snprintf(nm, sizeof nm, "p_%d", lev);
		rec_d(nm, p + 1, npno);
		assemble_grad_p(E, p, au, lev);
		snprintf(nm, sizeof nm, "gradp_%d", lev);
		rec_d(nm, au, neq);

		/* gauss_seidel from zero on a stripped right-hand side */
		{
			double *f = calloc(neq + 4, sizeof(double));
			double *d0 = calloc(neq + 4, sizeof(double));
			double *ad = calloc(neq + 4, sizeof(double));
			test_vector(f, neq, 0.19, 0.7);
			strip_bcs_from_residual(E, f, lev);
			snprintf(nm, sizeof nm, "gsF_%d", lev);
			rec_d(nm, f, neq);
			cycles = 2;
			gauss_seidel(E, d0, f, ad, 0.0, &cycles, lev, 0);
			snprintf(nm, sizeof nm, "gsd_%d", lev);
			rec_d(nm, d0, neq);
			snprintf(nm, sizeof nm, "gsAd_%d", lev);
			rec_d(nm, ad, neq);
			/* a second call that starts from the previous iterate */
			cycles = 1;
			gauss_seidel(E, d0, f, ad, 0.0, &cycles, lev, 1);
			snprintf(nm, sizeof nm, "gsd2_%d", lev);
			rec_d(nm, d0, neq);
			free(f);
			free(d0);
			free(ad);
		}

		if(lev > lmin)
		{
			const int neqc = E->lmesh.NEQ[lev - 1];
			double *ad = calloc(neqc + 4, sizeof(double));
			double *af = calloc(neq + 4, sizeof(double));
			test_vector(u, neq, 0.29, 0.3);
			project_vector(E, lev, u, ad, 1);
			snprintf(nm, sizeof nm, "proj_%d", lev);
			rec_d(nm, ad, neqc);
			test_vector(ad, neqc, 0.43, 0.9);
			interp_vector(E, lev - 1, ad, af);
			snprintf(nm, sizeof nm, "interp_%d", lev);
			rec_d(nm, af, neq);
			free(ad);
			free(af);
		}
		free(u);
		free(au);
		free(p);
		free(flags);
	}

	/* one full-multigrid pass and one solve_del2_u on the fine level */
	{
		const int neq = E->lmesh.NEQ[lmax];
		double *f = calloc(neq + 4, sizeof(double));
		double *d1 = calloc(neq + 4, sizeof(double));
		double *au = calloc(neq + 4, sizeof(double));
		double res;
		int i;
		for(i = 0; i < neq; i++)
			f[i] = E->F[i];
		rec_d("mgF", f, neq);
		res = multi_grid(E, d1, f, au, 1e-3, lmax);
		rec_d("mg_d1", d1, neq);
		rec_d("mg_res", f, neq);
		rec_s("mg_residual", res);
		for(i = 0; i < neq; i++)
			f[i] = E->F[i];
		for(i = 0; i < neq; i++)
			d1[i] = 0.0;
		i = solve_del2_u(E, d1, f, 1e-4 * sqrt(global_vdot(E, f, f, lmax) / neq), lmax);
		rec_d("sdu_d0", d1, neq);
		rec_s("sdu_valid", (double)i);
		free(f);
		free(d1);
		free(au);
	}
}

static double vrms_of(struct All_variables *E)
{
	/* sqrt of the volume average of |u|^2, 2x2x2 Gauss over Q1 elements */
	int e, k, a;
	double s = 0.0, vol = 0.0;
	for(e = 1; e <= E->lmesh.nel; e++)
		for(k = 1; k <= 8; k++)
		{
			double u1 = 0, u2 = 0, u3 = 0, w;
			for(a = 1; a <= 8; a++)
			{
				int n = E->ien[e].node[a];
				double N = E->N.vpt[GNVINDEX(a, k)];
				u1 += N * E->V[1][n];
				u2 += N * E->V[2][n];
				u3 += N * E->V[3][n];
			}
			w = E->gDA[e].vpt[k];
			s += w * (u1 * u1 + u2 * u2 + u3 * u3);
			vol += w;
		}
	return sqrt(s / vol);
}

/* The output-step fields after heat_flux: the layer profiles that
 * output_velo_related writes to the .ave file (Have.T, Rho, F, f from heat_flux;
 * Have.vrms and Have.Vi computed here as averages, Process_velocity.c:179-224,
 * does, through the same reference routines, without its composition part),
 * the nodal heatflux / heatflux_adv and the surface fluxes of the .th_t/.th_b
 * files. */
static void dump_output_fields(struct All_variables *E, int step)
{
	char nm[64];
	const int nno = E->lmesh.nno, noz = E->lmesh.noz, nsf = E->lmesh.nsf;
	const int lev = E->mesh.levmax;
	float *temp = (float *)malloc((size_t)(nno + 1) * sizeof(float));
	double *have = (double *)malloc((size_t)6 * noz * sizeof(double));
	double *surf = (double *)malloc((size_t)2 * nsf * sizeof(double));
	int i;
	visc_from_gint_to_nodes(E, E->EVI[lev], temp, lev);
	return_horiz_ave(E, temp, E->Have.Vi);
	for(i = 1; i <= nno; i++)
		temp[i] = E->V[1][i] * E->V[1][i] + E->V[2][i] * E->V[2][i] + E->V[3][i] * E->V[3][i];
	return_horiz_ave(E, temp, E->Have.vrms);
	for(i = 1; i <= noz; i++)
		E->Have.vrms[i] = sqrt(E->Have.vrms[i]);
	for(i = 0; i < noz; i++)
	{
		have[i] = E->Have.T[i + 1];
		have[noz + i] = E->Have.vrms[i + 1];
		have[2 * noz + i] = E->Have.Vi[i + 1];
		have[3 * noz + i] = E->Have.Rho[i + 1];
		have[4 * noz + i] = E->Have.F[i + 1];
		have[5 * noz + i] = E->Have.f[i + 1];
	}
	for(i = 0; i < nsf; i++)
	{
		surf[i] = E->slice.shflux[i + 1];
		surf[nsf + i] = E->slice.bhflux[i + 1];
	}
	snprintf(nm, sizeof nm, "s%d_Have", step);
	rec_d(nm, have, 6L * noz);
	snprintf(nm, sizeof nm, "s%d_surf", step);
	rec_d(nm, surf, 2L * nsf);
	snprintf(nm, sizeof nm, "s%d_heatflux", step);
	rec_f(nm, E->heatflux + 1, nno);
	snprintf(nm, sizeof nm, "s%d_heatflux_adv", step);
	rec_f(nm, E->heatflux_adv + 1, nno);
	free(temp);
	free(have);
	free(surf);
}

static void dump_state(struct All_variables *E, int step, double stokes_s, int uzawa_calls, int mg_cycles)
{
	char nm[64];
	const int nno = E->lmesh.nno, neq = E->lmesh.neq, npno = E->lmesh.npno;
	snprintf(nm, sizeof nm, "s%d_T", step);
	rec_f(nm, E->T + 1, nno);
	snprintf(nm, sizeof nm, "s%d_V1", step);
	rec_f(nm, E->V[1] + 1, nno);
	snprintf(nm, sizeof nm, "s%d_V2", step);
	rec_f(nm, E->V[2] + 1, nno);
	snprintf(nm, sizeof nm, "s%d_V3", step);
	rec_f(nm, E->V[3] + 1, nno);
	snprintf(nm, sizeof nm, "s%d_U", step);
	rec_d(nm, E->U, neq);
	snprintf(nm, sizeof nm, "s%d_P", step);
	rec_d(nm, E->P + 1, npno);
	snprintf(nm, sizeof nm, "s%d_F", step);
	rec_d(nm, E->F, neq);
	snprintf(nm, sizeof nm, "s%d_Tdot", step);
	rec_f(nm, E->Tdot + 1, nno);
	{
		double sc[10];
		sc[0] = E->slice.Nut;
		sc[1] = E->slice.Nub;
		sc[2] = vrms_of(E);
		sc[3] = E->advection.timestep;
		sc[4] = E->monitor.elapsed_time;
		sc[5] = stokes_s;
		sc[6] = uzawa_calls;
		sc[7] = mg_cycles;
		sc[8] = E->monitor.T_interior;
		sc[9] = E->advection.last_sub_iterations;
		snprintf(nm, sizeof nm, "s%d_scalars", step);
		rec_d(nm, sc, 10);
	}
	dump_output_fields(E, step);
}

static void timed_stokes(struct All_variables *E, double *secs, int *calls, int *cycles)
{
	int c0 = E->control.total_v_solver_calls;
	int i0 = E->control.total_iteration_cycles;
	double t0 = MPI_Wtime();
	general_stokes_solver(E);
	*secs = MPI_Wtime() - t0;
	*calls = E->control.total_v_solver_calls - c0;
	*cycles = E->control.total_iteration_cycles - i0;
}

int main(int argc, char **argv)
{
	struct All_variables E;
	double secs;
	int calls, cycles, nsteps, probe, step;
	char *rargv[2];

	if(argc < 5)
	{
		fprintf(stderr, "usage: %s deck T0.bin|- nsteps out.bin [probe]\n", argv[0]);
		return 2;
	}
	nsteps = atoi(argv[3]);
	probe = (argc > 5 && strcmp(argv[5], "probe") == 0);
	out = fopen(argv[4], "wb");
	if(!out)
	{
		perror(argv[4]);
		return 2;
	}

	memset(&E, 0, sizeof(E));
	srand48((long int)-1);
	E.parallel.me = 0;
	E.parallel.nproc = 1;
	E.parallel.me_loc[1] = E.parallel.me_loc[2] = E.parallel.me_loc[3] = 0;
	MPI_Init(&argc, &argv);
	E.monitor.solution_cycles = 0;
	E.monitor.elapsed_time = 0;
	E.advection.timestep = 0;
	E.advection.timesteps = 0;

	rargv[0] = argv[0];
	rargv[1] = argv[1];
	read_instructions(&E, 2, rargv);
	E.control.keep_going = 1;

	if(strcmp(argv[2], "-") != 0)
	{
		FILE *f = fopen(argv[2], "rb");
		double *t = (double *)malloc(sizeof(double) * (size_t)E.lmesh.nno);
		int i;
		if(!f || fread(t, sizeof(double), (size_t)E.lmesh.nno, f) != (size_t)E.lmesh.nno)
		{
			fprintf(stderr, "cannot read %d doubles from %s\n", E.lmesh.nno, argv[2]);
			return 2;
		}
		fclose(f);
		for(i = 1; i <= E.lmesh.nno; i++)
			E.T[i] = t[i - 1];
		free(t);
		temperatures_conform_bcs(&E);
		thermal_buoyancy(&E);
		if(E.viscosity.update_allowed)
			get_system_viscosity(&E, 1, E.EVI[E.mesh.levmax], E.VI[E.mesh.levmax]);
	}
	{
		double dims[8];
		dims[0] = E.mesh.levmin;
		dims[1] = E.mesh.levmax;
		dims[2] = E.lmesh.nox;
		dims[3] = E.lmesh.noy;
		dims[4] = E.lmesh.noz;
		dims[5] = E.lmesh.nno;
		dims[6] = E.lmesh.neq;
		dims[7] = E.lmesh.npno;
		rec_d("dims", dims, 8);
		rec_f("T0", E.T + 1, E.lmesh.nno);
		rec_f("X1", E.X[1] + 1, E.lmesh.nno);
		rec_f("X2", E.X[2] + 1, E.lmesh.nno);
		rec_f("X3", E.X[3] + 1, E.lmesh.nno);
		rec_f("buoyancy0", E.buoyancy + 1, E.lmesh.nno);
	}

	timed_stokes(&E, &secs, &calls, &cycles);
	process_temp_field(&E, E.monitor.solution_cycles);
	dump_state(&E, 0, secs, calls, cycles);
	if(probe)
		probe_operators(&E);

	for(step = 1; step <= nsteps && E.control.keep_going; step++)
	{
		if(E.control.composition != 2)
			process_heating(&E);
		E.monitor.solution_cycles++;
		if(E.monitor.solution_cycles > E.control.print_convergence)
			E.control.print_convergence = 1;
		(E.next_buoyancy_field) (&E);
		process_temp_field(&E, E.monitor.solution_cycles);
		timed_stokes(&E, &secs, &calls, &cycles);
		/* Nu of the new (T, V) pair, so that the record is self-consistent */
		heat_flux(&E);
		dump_state(&E, step, secs, calls, cycles);
		fflush(out);
	}
	fclose(out);
	return 0;
}
