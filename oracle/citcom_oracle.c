/*
 * CPU restatement of CitcomCU's Stokes / SUPG hot path.  TEST INFRASTRUCTURE:
 * the checker for the GPU library, never part of it.  See citcom_oracle.h.
 *
 * Scope: Cartesian box (CART3D), uniform spacing per axis on every multigrid
 * level, free-slip walls with the reference's default reflecting sides,
 * T fixed at top and bottom, insulating sides, one MPI rank.  All arithmetic
 * in FP64 (the reference stores several of these arrays in FP32; the
 * comparison is against the reference compiled with -Dfloat=double).
 */
#include "citcom_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NL ORACLE_MAX_LEVELS

/* local node a (0..7) -> (x, y, z) offsets; same sign pattern for the
 * 2x2x2 Gauss points (element_definitions.h:139-179, bb[] at :233-235,
 * offset[] at :214-222) */
static const int LOC[8][3] = {
	{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
	{0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

typedef struct level
{
	int nox, noy, noz, nno, nel, neq, elx, ely, elz;
	double h[3];          /* element edge lengths x, y, z */
	double J;             /* |dx/dxi| = hx*hy*hz/8, same at every point */
	double gnx[8][8][3];  /* dN_a/dx_d at Gauss point k: [k][a][d] */
	double gnxc[8][3];    /* dN_a/dx_d at the element centre */
	double g[24];         /* divergence operator of one element (get_elt_g) */
	double *evi;          /* viscosity at the 8 Gauss points of each element */
	double *K;            /* assembled block stencil: node*243 + slot*9 + 3i + j */
	double *H;            /* half stencil of the reference (construct_node_maps): per node the
	                         self block and the 13 lower-numbered neighbours' blocks, 14*9 words,
	                         with the neighbour index of each block in HI */
	int *HI;
	double *BI;           /* 1 / diag(K) (unmasked) */
	double *BPI;          /* pressure preconditioner */
	double *mass;         /* 1 / lumped mass */
	unsigned *vflag;      /* velocity BC bits */
} level;

struct oracle
{
	oracle_params p;
	int L;
	level lv[NL];
	double Nv[8][8];      /* N_a at Gauss point k: [k][a] */
	double *T, *Tdot, *V[3], *U, *P, *F, *buoy;
	unsigned *tflag;      /* Dirichlet temperature at the fine level */
	int *mat;             /* material group (0-based) of fine elements */
	double timestep, elapsed, T_interior;
	/* multi_grid work (General_matrix_functions.c:545-557) */
	double *vel[NL], *res[NL], *rhs[NL], *fl[NL], *del_vel[NL], *AU[NL];
	/* solve_del2_u work (General_matrix_functions.c:376-384) */
	double *sr, *sD1, *sAu;
	/* solve_Ahat_p_fhat work (Stokes_flow_Incomp.c:323-336) */
	double *r0, *r1, *r2, *z0, *z1, *s1, *s2, *Ah, *u1;
	double *gs_tmp;
	/* stress-dependent viscosity: the previous solution of the viscosity
	   iteration (static oldU of general_stokes_solver), the element strain
	   rates, and how often visc_from_S ran (its static `visits`) */
	double *oldU, *edot;
	int sdepv_visits;
	/* the residual rule's last momentum and continuity residuals and its
	   velocity corrections */
	double last_momentum, last_continuity;
	int last_corrections;
};

static void *xcalloc(size_t n, size_t s)
{
	void *p = calloc(n ? n : 1, s);
	if(!p)
	{
		fprintf(stderr, "oracle: out of memory\n");
		abort();
	}
	return p;
}

static inline int nidx(const level *l, int x, int y, int z) { return z + x * l->noz + y * l->noz * l->nox; }
static inline int eidx(const level *l, int x, int y, int z) { return z + x * l->elz + y * l->elz * l->elx; }

/* nodes of element e in local order */
static void elem_nodes(const level *l, int e, int nodes[8])
{
	int ez = e % l->elz, ex = (e / l->elz) % l->elx, ey = e / (l->elz * l->elx);
	int a;
	for(a = 0; a < 8; a++)
		nodes[a] = nidx(l, ex + LOC[a][0], ey + LOC[a][1], ez + LOC[a][2]);
}

static inline int slot_of(int dx, int dy, int dz) { return (dz + 1) + 3 * (dx + 1) + 9 * (dy + 1); }

/* ---------------------------------------------------------------- set-up */

/* shape functions: construct_shape_functions (Shape_functions.c:53-168) and
 * the box-element case of get_global_shape_fn (Size_does_matter.c:60-179) */
static void setup_geometry(oracle *o)
{
	const double beta = 0.57735026918962576451;
	int l, k, a, d;
	for(k = 0; k < 8; k++)
		for(a = 0; a < 8; a++)
		{
			double v = 1.0;
			for(d = 0; d < 3; d++)
			{
				double sa = LOC[a][d] ? 1.0 : -1.0, sk = LOC[k][d] ? 1.0 : -1.0;
				v *= 0.5 * (1.0 + sa * sk * beta);
			}
			o->Nv[k][a] = v;
		}
	for(l = 0; l < o->L; l++)
	{
		level *lv = &o->lv[l];
		lv->J = lv->h[0] * lv->h[1] * lv->h[2] / 8.0;
		for(k = 0; k <= 8; k++)
			for(a = 0; a < 8; a++)
				for(d = 0; d < 3; d++)
				{
					/* k == 8 is the centre (pressure point) */
					double v = 0.5 * (LOC[a][d] ? 1.0 : -1.0) * 2.0 / lv->h[d];
					int dd;
					for(dd = 0; dd < 3; dd++)
						if(dd != d)
						{
							double sa = LOC[a][dd] ? 1.0 : -1.0;
							double xi = (k == 8) ? 0.0 : (LOC[k][dd] ? beta : -beta);
							v *= 0.5 * (1.0 + sa * xi);
						}
					if(k == 8)
						lv->gnxc[a][d] = v;
					else
						lv->gnx[k][a][d] = v;
				}
		/* get_elt_g (Element_calculations.c:831-934), Cartesian: g = -dN/dx * 8 * |J| at the centre */
		for(a = 0; a < 8; a++)
			for(d = 0; d < 3; d++)
				lv->g[3 * a + d] = -lv->gnxc[a][d] * 8.0 * lv->J;
	}
}

/* velocity BC bits per level: free slip on top/bottom (Boundary_conditions.c:
 * 44-73) combined with the default reflecting side walls (:249-370): a dof is
 * constrained exactly on the walls normal to it */
static void setup_flags(oracle *o)
{
	int l, x, y, z;
	for(l = 0; l < o->L; l++)
	{
		level *lv = &o->lv[l];
		for(y = 0; y < lv->noy; y++)
			for(x = 0; x < lv->nox; x++)
				for(z = 0; z < lv->noz; z++)
				{
					unsigned f = 0;
					if(x == 0 || x == lv->nox - 1)
						f |= 1u;
					if(y == 0 || y == lv->noy - 1)
						f |= 2u;
					if(z == 0 || z == lv->noz - 1)
						f |= 4u;
					lv->vflag[nidx(lv, x, y, z)] = f;
				}
	}
	{
		level *lv = &o->lv[o->L - 1];
		for(y = 0; y < lv->noy; y++)
			for(x = 0; x < lv->nox; x++)
				for(z = 0; z < lv->noz; z++)
					o->tflag[nidx(lv, x, y, z)] = (z == 0 || z == lv->noz - 1) ? 1u : 0u;
	}
}

/* lumped mass: mass_matrix (Size_does_matter.c:618-757); MASS = 1/sum(TWW), TWW = |J| */
static void setup_mass(oracle *o)
{
	int l, e, a, n[8];
	for(l = 0; l < o->L; l++)
	{
		level *lv = &o->lv[l];
		for(a = 0; a < lv->nno; a++)
			lv->mass[a] = 0.0;
		for(e = 0; e < lv->nel; e++)
		{
			elem_nodes(lv, e, n);
			for(a = 0; a < 8; a++)
				lv->mass[n[a]] += lv->J;
		}
		for(a = 0; a < lv->nno; a++)
			lv->mass[a] = 1.0 / lv->mass[a];
	}
}

/* construct_mat_group (Construct_arrays.c:742-800) with layers()
 * (Viscosity_structures.c:1389-1403) */
static void setup_materials(oracle *o)
{
	level *lv = &o->lv[o->L - 1];
	int e, n[8], a, i;
	for(e = 0; e < lv->nel; e++)
	{
		double zc = 0.0;
		int layer = 0;
		elem_nodes(lv, e, n);
		for(a = 0; a < 8; a++)
			zc += (double)(n[a] % lv->noz) * lv->h[2];
		zc /= 8.0;
		for(i = 0; i < o->p.num_mat - 1; i++)
			if(zc >= o->p.z_layer[i])
			{
				layer = i + 1;
				break;
			}
		if(!layer)
			layer = o->p.num_mat;
		o->mat[e] = layer - 1;
	}
}

oracle *oracle_create(const oracle_params *p)
{
	oracle *o = (oracle *)xcalloc(1, sizeof(oracle));
	int l;
	o->p = *p;
	o->L = p->levels;
	for(l = 0; l < o->L; l++)
	{
		level *lv = &o->lv[l];
		lv->nox = p->mgunit[0] * (1 << l) + 1;
		lv->noy = p->mgunit[1] * (1 << l) + 1;
		lv->noz = p->mgunit[2] * (1 << l) + 1;
		lv->elx = lv->nox - 1;
		lv->ely = lv->noy - 1;
		lv->elz = lv->noz - 1;
		lv->nno = lv->nox * lv->noy * lv->noz;
		lv->nel = lv->elx * lv->ely * lv->elz;
		lv->neq = 3 * lv->nno;
		lv->h[0] = p->dimen[0] / lv->elx;
		lv->h[1] = p->dimen[1] / lv->ely;
		lv->h[2] = p->dimen[2] / lv->elz;
		lv->evi = (double *)xcalloc((size_t)lv->nel * 8, sizeof(double));
		lv->K = (double *)xcalloc((size_t)lv->nno * 243, sizeof(double));
		lv->H = (double *)xcalloc((size_t)lv->nno * 126, sizeof(double));
		lv->HI = (int *)xcalloc((size_t)lv->nno * 14, sizeof(int));
		lv->BI = (double *)xcalloc((size_t)lv->neq + 2, sizeof(double));
		lv->BPI = (double *)xcalloc((size_t)lv->nel, sizeof(double));
		lv->mass = (double *)xcalloc((size_t)lv->nno, sizeof(double));
		lv->vflag = (unsigned *)xcalloc((size_t)lv->nno, sizeof(unsigned));
		o->vel[l] = (double *)xcalloc((size_t)lv->neq + 2, sizeof(double));
		o->res[l] = (double *)xcalloc((size_t)lv->neq + 2, sizeof(double));
		o->rhs[l] = (double *)xcalloc((size_t)lv->neq + 2, sizeof(double));
		o->fl[l] = (double *)xcalloc((size_t)lv->neq + 2, sizeof(double));
		o->del_vel[l] = (double *)xcalloc((size_t)lv->neq + 2, sizeof(double));
		o->AU[l] = (double *)xcalloc((size_t)lv->neq + 2, sizeof(double));
	}
	{
		level *f = &o->lv[o->L - 1];
		int d;
		o->T = (double *)xcalloc(f->nno, sizeof(double));
		o->Tdot = (double *)xcalloc(f->nno, sizeof(double));
		for(d = 0; d < 3; d++)
			o->V[d] = (double *)xcalloc(f->nno, sizeof(double));
		o->U = (double *)xcalloc(f->neq + 2, sizeof(double));
		o->P = (double *)xcalloc(f->nel, sizeof(double));
		o->F = (double *)xcalloc(f->neq + 2, sizeof(double));
		o->buoy = (double *)xcalloc(f->nno, sizeof(double));
		o->tflag = (unsigned *)xcalloc(f->nno, sizeof(unsigned));
		o->mat = (int *)xcalloc(f->nel, sizeof(int));
		o->sr = (double *)xcalloc(f->neq + 10, sizeof(double));
		o->sD1 = (double *)xcalloc(f->neq + 10, sizeof(double));
		o->sAu = (double *)xcalloc(f->neq + 10, sizeof(double));
		o->r0 = (double *)xcalloc(f->nel, sizeof(double));
		o->r1 = (double *)xcalloc(f->nel, sizeof(double));
		o->r2 = (double *)xcalloc(f->nel, sizeof(double));
		o->z0 = (double *)xcalloc(f->nel, sizeof(double));
		o->z1 = (double *)xcalloc(f->nel, sizeof(double));
		o->s1 = (double *)xcalloc(f->nel, sizeof(double));
		o->s2 = (double *)xcalloc(f->nel, sizeof(double));
		o->Ah = (double *)xcalloc(f->neq + 2, sizeof(double));
		o->u1 = (double *)xcalloc(f->neq + 2, sizeof(double));
		o->gs_tmp = (double *)xcalloc(f->neq + 2, sizeof(double));
		o->oldU = (double *)xcalloc(f->neq + 2, sizeof(double));
		o->edot = (double *)xcalloc(f->nel + 1, sizeof(double));
	}
	setup_geometry(o);
	setup_flags(o);
	setup_mass(o);
	setup_materials(o);
	/* isoviscous default until the caller asks for get_system_viscosity */
	{
		level *f = &o->lv[o->L - 1];
		int e, k;
		for(e = 0; e < f->nel; e++)
			for(k = 0; k < 8; k++)
				f->evi[8 * e + k] = o->p.visc0[o->mat[e]];
	}
	return o;
}

void oracle_destroy(oracle *o)
{
	int l, d;
	if(!o)
		return;
	for(l = 0; l < o->L; l++)
	{
		level *lv = &o->lv[l];
		free(lv->evi);
		free(lv->K);
		free(lv->H);
		free(lv->HI);
		free(lv->BI);
		free(lv->BPI);
		free(lv->mass);
		free(lv->vflag);
		free(o->vel[l]);
		free(o->res[l]);
		free(o->rhs[l]);
		free(o->fl[l]);
		free(o->del_vel[l]);
		free(o->AU[l]);
	}
	free(o->T);
	free(o->Tdot);
	for(d = 0; d < 3; d++)
		free(o->V[d]);
	free(o->U);
	free(o->P);
	free(o->F);
	free(o->buoy);
	free(o->tflag);
	free(o->mat);
	free(o->sr);
	free(o->sD1);
	free(o->sAu);
	free(o->r0);
	free(o->r1);
	free(o->r2);
	free(o->z0);
	free(o->z1);
	free(o->s1);
	free(o->s2);
	free(o->Ah);
	free(o->u1);
	free(o->gs_tmp);
	free(o->oldU);
	free(o->edot);
	free(o);
}

void oracle_level_dims(const oracle *o, int lev, int dims[6])
{
	const level *l = &o->lv[lev];
	dims[0] = l->nox;
	dims[1] = l->noy;
	dims[2] = l->noz;
	dims[3] = l->nno;
	dims[4] = l->nel;
	dims[5] = l->neq;
}

double *oracle_T(oracle *o) { return o->T; }
double *oracle_Tdot(oracle *o) { return o->Tdot; }
double *oracle_U(oracle *o) { return o->U; }
double *oracle_P(oracle *o) { return o->P; }
double *oracle_F(oracle *o) { return o->F; }
double *oracle_V(oracle *o, int d) { return o->V[d]; }
double *oracle_buoyancy(oracle *o) { return o->buoy; }
double *oracle_EVI(oracle *o, int lev) { return o->lv[lev].evi; }
double *oracle_BI(oracle *o, int lev) { return o->lv[lev].BI; }
double *oracle_BPI(oracle *o, int lev) { return o->lv[lev].BPI; }
unsigned *oracle_vflags(oracle *o, int lev) { return o->lv[lev].vflag; }
double *oracle_stencil(oracle *o, int lev) { return o->lv[lev].K; }
double oracle_timestep(const oracle *o) { return o->timestep; }
double oracle_elapsed_time(const oracle *o) { return o->elapsed; }
double oracle_T_interior(const oracle *o) { return o->T_interior; }
void oracle_set_timestep(oracle *o, double dt) { o->timestep = dt; }

/* ------------------------------------------------------ horizontal means */

/* return_horiz_ave (Global_operations.c:133-251) for a box grid: per z layer
 * the area-weighted mean of the bilinear interpolant, i.e. sum over the
 * horizontal elements of (area/4) * (sum of its 4 nodal values) divided by the
 * layer area */
static void horiz_ave(const oracle *o, const double *X, double *H)
{
	const level *f = &o->lv[o->L - 1];
	int z, x, y;
	for(z = 0; z < f->noz; z++)
	{
		double s = 0.0, w = 0.0;
		for(y = 0; y < f->ely; y++)
			for(x = 0; x < f->elx; x++)
			{
				double dg = f->h[0] * f->h[1] / 4.0;
				s += dg * (X[nidx(f, x, y, z)] + X[nidx(f, x + 1, y, z)] + X[nidx(f, x + 1, y + 1, z)] + X[nidx(f, x, y + 1, z)]);
				w += 4.0 * dg;
			}
		H[z] = s / w;
	}
}

/* thermal_buoyancy (Pan_problem_misc_functions.c:83-156), thermal only,
 * expansivity 1: buoyancy = Ra*T minus its horizontal average */
void oracle_thermal_buoyancy(oracle *o)
{
	const level *f = &o->lv[o->L - 1];
	double *H = (double *)xcalloc(f->noz, sizeof(double));
	int n;
	for(n = 0; n < f->nno; n++)
		o->buoy[n] = o->p.rayleigh * o->T[n];
	horiz_ave(o, o->buoy, H);
	for(n = 0; n < f->nno; n++)
		o->buoy[n] -= H[n % f->noz];
	free(H);
}

/* strip_bcs_from_residual (Boundary_conditions.c:926-945) */
void oracle_strip_bcs(oracle *o, int lev, double *r)
{
	const level *l = &o->lv[lev];
	int n, d;
	for(n = 0; n < l->nno; n++)
		for(d = 0; d < 3; d++)
			if(l->vflag[n] & (1u << d))
				r[3 * n + d] = 0.0;
}

/* assemble_forces (Element_calculations.c:74-125) with get_elt_f (:989-1075),
 * Cartesian branch; imposed velocities are zero for free slip */
void oracle_assemble_forces(oracle *o)
{
	const level *f = &o->lv[o->L - 1];
	int e, a, k, b, n[8];
	for(a = 0; a < f->neq + 2; a++)
		o->F[a] = 0.0;
	for(e = 0; e < f->nel; e++)
	{
		double fgs[8];
		elem_nodes(f, e, n);
		for(k = 0; k < 8; k++)
		{
			fgs[k] = 0.0;
			for(b = 0; b < 8; b++)
				fgs[k] += o->buoy[n[b]] * o->Nv[k][b];
		}
		for(a = 0; a < 8; a++)
		{
			double s = 0.0;
			for(k = 0; k < 8; k++)
				s += fgs[k] * o->Nv[k][a] * f->J;
			o->F[3 * n[a] + 2] += s;
		}
	}
	oracle_strip_bcs(o, o->L - 1, o->F);
}

/* ------------------------------------------------------------- viscosity */

/* strain_rate_2_inv (Viscosity_structures.c:979-1086), Cartesian branch
 * (:1042-1075) with SQRT: per element the symmetric velocity gradient at the
 * centre from V, edot = sqrt(0.5 (e11^2 + e22^2 + e33^2 + 2 e12^2 + 2 e13^2
 * + 2 e23^2)) */
static void strain_rate(oracle *o, double *edot)
{
	const level *f = &o->lv[o->L - 1];
	int e, a, p, q, n[8];
	for(e = 0; e < f->nel; e++)
	{
		double du[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, ed[3][3];
		elem_nodes(f, e, n);
		for(a = 0; a < 8; a++)
			for(p = 0; p < 3; p++)
				for(q = 0; q < 3; q++)
					du[p][q] += o->V[p][n[a]] * f->gnxc[a][q];
		for(p = 0; p < 3; p++)
			for(q = 0; q < 3; q++)
				ed[p][q] = 0.5 * (du[p][q] + du[q][p]);
		edot[e] = sqrt(0.5 * (ed[0][0] * ed[0][0] + ed[0][1] * ed[0][1] * 2.0 + ed[1][1] * ed[1][1] +
		                      ed[1][2] * ed[1][2] * 2.0 + ed[2][2] * ed[2][2] + ed[0][2] * ed[0][2] * 2.0));
	}
}

/* visc_from_S (Viscosity_structures.c:744-846), rheologies 1 and 2: with
 * s = (2 edot / trns)^(1 - 1/n) of the element's material, eta <- 2 eta /
 * (1 + s eta^(1-1/n)) (1) or eta <- eta / (1 + s eta^(1-1/n)) where the
 * Gauss-point temperature is below the transition temperature (2; the
 * reference's default transition values 3000 for T and 2 for the absent
 * composition are always above).  The first visit without a restart uses a
 * unit strain rate (:787-790). */
static void visc_from_S(oracle *o)
{
	level *f = &o->lv[o->L - 1];
	int e, k, a, n[8];
	if(o->sdepv_visits == 0)
		for(e = 0; e < f->nel; e++)
			o->edot[e] = 1.0;
	else
		strain_rate(o, o->edot);
	for(e = 0; e < f->nel; e++)
	{
		const int m = o->mat[e];
		const double e1 = 1.0 - 1.0 / o->p.sdepv_expt[m];
		const double scale = pow(2.0 * o->edot[e] / o->p.sdepv_trns[m], e1);
		elem_nodes(f, e, n);
		for(k = 0; k < 8; k++)
		{
			double v = f->evi[8 * e + k];
			if(o->p.sdepv_rheology == 1)
				v = 2.0 * v / (1.0 + scale * pow(v, e1));
			else
			{
				double t = 0.0;
				for(a = 0; a < 8; a++)
					t += (o->T[n[a]] > 0.0 ? o->T[n[a]] : 0.0) * o->Nv[k][a];
				if(t < 3000.0)
					v = v / (1.0 + scale * pow(v, e1));
			}
			f->evi[8 * e + k] = v;
		}
	}
	o->sdepv_visits++;
}

/* get_system_viscosity (Viscosity_structures.c:369-455): visc_from_T rheol 3
 * (:617-646) when TDEPV, else visc_from_mat (:477-489); visc_from_S when
 * SDEPV; then VMAX/VMIN (:414-427) */
void oracle_get_system_viscosity(oracle *o)
{
	level *f = &o->lv[o->L - 1];
	int e, k, a, n[8];
	for(e = 0; e < f->nel; e++)
	{
		int m = o->mat[e];
		elem_nodes(f, e, n);
		for(k = 0; k < 8; k++)
		{
			double v;
			if(o->p.tdepv)
			{
				double t = 1.0e-32;
				for(a = 0; a < 8; a++)
					t += (o->T[n[a]] > 0.0 ? o->T[n[a]] : 0.0) * o->Nv[k][a];
				v = o->p.visc0[m] * exp(o->p.viscE[m] * (o->p.viscT[m] - t));
			}
			else
				v = o->p.visc0[m];
			f->evi[8 * e + k] = v;
		}
	}
	if(o->p.sdepv)
		visc_from_S(o);
	for(e = 0; e < 8 * f->nel; e++)
	{
		if(o->p.vmax_on && f->evi[e] > o->p.vmax)
			f->evi[e] = o->p.vmax;
		if(o->p.vmin_on && f->evi[e] < o->p.vmin)
			f->evi[e] = o->p.vmin;
	}
}

/* project_viscosity (Solver_multigrid.c:398-480) with visc_smooth_cycles=1:
 * visc_from_gint_to_nodes (Nodal_mesh.c:583-615), project_scalar
 * (Solver_multigrid.c:338-394), visc_from_nodes_to_gint (Nodal_mesh.c:617-640) */
void oracle_project_viscosity(oracle *o)
{
	int lv;
	for(lv = o->L - 1; lv > 0; lv--)
	{
		level *F = &o->lv[lv], *C = &o->lv[lv - 1];
		double *VN = (double *)xcalloc(F->nno, sizeof(double));
		double *VD = (double *)xcalloc(C->nno, sizeof(double));
		int e, a, k, n[8], cn[8];
		for(e = 0; e < F->nel; e++)
		{
			double t = 0.0;
			for(k = 0; k < 8; k++)
				t += F->evi[8 * e + k];
			t /= 8.0;
			elem_nodes(F, e, n);
			for(a = 0; a < 8; a++)
				VN[n[a]] += F->J * t;
		}
		for(a = 0; a < F->nno; a++)
			VN[a] *= F->mass[a];
		for(e = 0; e < C->nel; e++)
		{
			int ez = e % C->elz, ex = (e / C->elz) % C->elx, ey = e / (C->elz * C->elx);
			elem_nodes(C, e, cn);
			for(a = 0; a < 8; a++)
			{
				int fe = eidx(F, 2 * ex + LOC[a][0], 2 * ey + LOC[a][1], 2 * ez + LOC[a][2]);
				double s = 0.0;
				int j;
				elem_nodes(F, fe, n);
				for(j = 0; j < 8; j++)
					s += VN[n[j]];
				VD[cn[a]] += (s / 8.0) * C->J;
			}
		}
		for(a = 0; a < C->nno; a++)
			VD[a] *= C->mass[a];
		for(e = 0; e < C->nel; e++)
		{
			elem_nodes(C, e, cn);
			for(k = 0; k < 8; k++)
			{
				double t = 0.0;
				for(a = 0; a < 8; a++)
					t += o->Nv[k][a] * VD[cn[a]];
				C->evi[8 * e + k] = t;
			}
		}
		free(VN);
		free(VD);
	}
}

/* ------------------------------------------------------------- stiffness */

/* get_elt_k Cartesian isotropic branch (Element_calculations.c:133-293)
 * plus get_aug_k (:1127-1163) */
static void elt_k(const oracle *o, const level *l, int e, double K[24][24])
{
	double W[8];
	int k, a, b, i, j, d;
	for(k = 0; k < 8; k++)
		W[k] = l->J * l->evi[8 * e + k];
	for(a = 0; a < 8; a++)
		for(b = 0; b < 8; b++)
			for(i = 0; i < 3; i++)
				for(j = 0; j < 3; j++)
				{
					double s = 0.0;
					for(k = 0; k < 8; k++)
					{
						double t = l->gnx[k][a][j] * l->gnx[k][b][i];
						if(i == j)
							for(d = 0; d < 3; d++)
								t += l->gnx[k][a][d] * l->gnx[k][b][d];
						s += W[k] * t;
					}
					K[3 * a + i][3 * b + j] = s;
				}
	if(o->p.aug_lagr)
	{
		double visc = 0.0;
		for(k = 0; k < 8; k++)
			visc += l->evi[8 * e + k];
		visc /= 8.0;
		for(a = 0; a < 24; a++)
			for(b = 0; b < 24; b++)
				K[a][b] += visc * o->p.aug_number * l->g[a] * l->g[b];
	}
}

/* construct_node_ks (Construct_arrays.c:359-535) as a full 27-block stencil
 * (the reference stores the symmetric lower half, construct_node_maps :280-356),
 * build_diagonal_of_K (Element_calculations.c:624-652) and
 * build_diagonal_of_Ahat / assemble_dAhatp_entry (:654-689, :771-829) */
void oracle_construct_stiffness(oracle *o)
{
	int lev;
	double K[24][24];
	for(lev = 0; lev < o->L; lev++)
	{
		level *l = &o->lv[lev];
		int e, a, b, i, j, n[8];
		memset(l->K, 0, sizeof(double) * (size_t)l->nno * 243);
		memset(l->BI, 0, sizeof(double) * (size_t)(l->neq + 2));
		for(e = 0; e < l->nel; e++)
		{
			elt_k(o, l, e, K);
			elem_nodes(l, e, n);
			for(a = 0; a < 8; a++)
			{
				for(i = 0; i < 3; i++)
					l->BI[3 * n[a] + i] += K[3 * a + i][3 * a + i];
				for(b = 0; b < 8; b++)
				{
					int s = slot_of(LOC[b][0] - LOC[a][0], LOC[b][1] - LOC[a][1], LOC[b][2] - LOC[a][2]);
					double *blk = l->K + (size_t)n[a] * 243 + 9 * s;
					for(i = 0; i < 3; i++)
					{
						if(l->vflag[n[a]] & (1u << i))
							continue;
						for(j = 0; j < 3; j++)
						{
							if(l->vflag[n[b]] & (1u << j))
								continue;
							blk[3 * i + j] += K[3 * a + i][3 * b + j];
						}
					}
				}
			}
		}
		for(i = 0; i < l->neq; i++)
			l->BI[i] = 1.0 / l->BI[i];
		/* half stencil in the order of construct_node_maps (Construct_arrays.c:280-356):
		   self first, then the neighbours with smaller node number, y-1 plane, x-1 row, z-1 */
		{
			int n;
			for(n = 0; n < l->nno; n++)
			{
				int z = n % l->noz, x = (n / l->noz) % l->nox, y = n / (l->noz * l->nox);
				int dx, dy, dz, cnt = 0, q;
				for(q = 0; q < 14; q++)
					l->HI[14 * n + q] = -1;
				memcpy(l->H + (size_t)126 * n, l->K + (size_t)243 * n + 9 * slot_of(0, 0, 0), 9 * sizeof(double));
				l->HI[14 * n] = n;
				cnt = 1;
				for(dy = -1; dy <= 0; dy++)
					for(dx = -1; dx <= 1; dx++)
						for(dz = -1; dz <= 1; dz++)
						{
							if(dy == 0 && (dx > 0 || (dx == 0 && dz >= 0)))
								continue;
							if(y + dy < 0 || x + dx < 0 || x + dx >= l->nox || z + dz < 0 || z + dz >= l->noz)
								continue;
							memcpy(l->H + (size_t)126 * n + 9 * cnt, l->K + (size_t)243 * n + 9 * slot_of(dx, dy, dz),
							       9 * sizeof(double));
							l->HI[14 * n + cnt] = nidx(l, x + dx, y + dy, z + dz);
							cnt++;
						}
			}
		}
		for(e = 0; e < l->nel; e++)
		{
			l->BPI[e] = 1.0;
			if(o->p.precond)
			{
				double bu = 0.0;
				elem_nodes(l, e, n);
				for(a = 0; a < 8; a++)
					for(i = 0; i < 3; i++)
						bu += l->g[3 * a + i] * l->g[3 * a + i] * l->BI[3 * n[a] + i];
				l->BPI[e] = (bu != 0.0) ? 1.0 / bu : 1.0;
			}
		}
	}
}

/* ------------------------------------------------------------- operators */

/* row product of node n: out[i] = sum over neighbours m of K_{n,m} u_m */
static inline void row_mul(const level *l, int n, const double *u, double out[3])
{
	int z = n % l->noz, x = (n / l->noz) % l->nox, y = n / (l->noz * l->nox);
	int dx, dy, dz;
	const double *Kn = l->K + (size_t)n * 243;
	out[0] = out[1] = out[2] = 0.0;
	for(dy = -1; dy <= 1; dy++)
	{
		if(y + dy < 0 || y + dy >= l->noy)
			continue;
		for(dx = -1; dx <= 1; dx++)
		{
			if(x + dx < 0 || x + dx >= l->nox)
				continue;
			for(dz = -1; dz <= 1; dz++)
			{
				const double *blk;
				const double *um;
				int m;
				if(z + dz < 0 || z + dz >= l->noz)
					continue;
				m = nidx(l, x + dx, y + dy, z + dz);
				blk = Kn + 9 * slot_of(dx, dy, dz);
				um = u + 3 * m;
				out[0] += blk[0] * um[0] + blk[1] * um[1] + blk[2] * um[2];
				out[1] += blk[3] * um[0] + blk[4] * um[1] + blk[5] * um[2];
				out[2] += blk[6] * um[0] + blk[7] * um[1] + blk[8] * um[2];
			}
		}
	}
}

/* n_assemble_del2_u (Element_calculations.c:552-621): in the reference's
 * order, each node gathers its lower neighbours' contributions and scatters
 * its own value through the transposed blocks of its half stencil; in the
 * colour mode (the GPU's arithmetic) every row is a full 27-block gather */
void oracle_kmul(oracle *o, int lev, const double *u, double *Au, int strip)
{
	const level *l = &o->lv[lev];
	int n;
	if(!o->p.gs_colored)
	{
		int i, q;
		for(i = 0; i < l->neq; i++)
			Au[i] = 0.0;
		for(n = 0; n < l->nno; n++)
		{
			const double *Hn = l->H + (size_t)126 * n;
			const int *In = l->HI + 14 * n;
			const double u0 = u[3 * n], u1 = u[3 * n + 1], u2 = u[3 * n + 2];
			for(q = 1; q < 14; q++)
			{
				const int m = In[q];
				const double *b = Hn + 9 * q;
				if(m < 0)
					break;
				Au[3 * n] += b[0] * u[3 * m] + b[1] * u[3 * m + 1] + b[2] * u[3 * m + 2];
				Au[3 * n + 1] += b[3] * u[3 * m] + b[4] * u[3 * m + 1] + b[5] * u[3 * m + 2];
				Au[3 * n + 2] += b[6] * u[3 * m] + b[7] * u[3 * m + 1] + b[8] * u[3 * m + 2];
			}
			for(q = 0; q < 14; q++)
			{
				const int m = In[q];
				const double *b = Hn + 9 * q;
				if(m < 0)
					break;
				Au[3 * m] += b[0] * u0 + b[3] * u1 + b[6] * u2;
				Au[3 * m + 1] += b[1] * u0 + b[4] * u1 + b[7] * u2;
				Au[3 * m + 2] += b[2] * u0 + b[5] * u1 + b[8] * u2;
			}
		}
		Au[l->neq] = Au[l->neq + 1] = 0.0;
		if(strip)
			oracle_strip_bcs(o, lev, Au);
		return;
	}
	for(n = 0; n < l->nno; n++)
		row_mul(l, n, u, Au + 3 * n);
	Au[l->neq] = Au[l->neq + 1] = 0.0;
	if(strip)
		oracle_strip_bcs(o, lev, Au);
}

/* gauss_seidel (General_matrix_functions.c:1160-1361), dims == 3, one rank.
 * Lexicographic mode keeps Ad = K d up to date exactly as the reference does:
 * the increments of lower-numbered neighbours are gathered into Ad_n, the
 * node's 3 dofs are relaxed together with the diagonal BI ("Jacobi at a
 * node"), and the node's increment is scattered into Ad of itself and its
 * lower neighbours.  Coloured mode relaxes the 8 parity classes of nodes in
 * turn from a full row product (what the GPU does) and forms Ad = K d at the
 * end. */
void oracle_gauss_seidel(oracle *o, int lev, double *d0, const double *F, double *Ad, int cycles, int guess)
{
	const level *l = &o->lv[lev];
	const int neq = l->neq;
	int i, c;
	double *temp = o->gs_tmp;
	if(guess)
	{
		d0[neq] = 0.0;
		oracle_kmul(o, lev, d0, Ad, 1);
	}
	else
		for(i = 0; i < neq; i++)
			d0[i] = Ad[i] = 0.0;

	for(c = 0; c < cycles; c++)
	{
		if(!o->p.gs_colored)
		{
			int n, q, d;
			for(i = 0; i <= neq + 1; i++)
				temp[i] = 0.0;
			for(n = 0; n < l->nno; n++)
			{
				const double *Hn = l->H + (size_t)126 * n;
				const int *In = l->HI + 14 * n;
				double t[3];
				/* gather lower neighbours' fresh increments: K_{n,m} temp_m */
				for(q = 1; q < 14; q++)
				{
					const int m = In[q];
					const double *b = Hn + 9 * q;
					if(m < 0)
						break;
					for(d = 0; d < 3; d++)
						Ad[3 * n + d] += b[3 * d] * temp[3 * m] + b[3 * d + 1] * temp[3 * m + 1] + b[3 * d + 2] * temp[3 * m + 2];
				}
				for(d = 0; d < 3; d++)
					t[d] = temp[3 * n + d] = (F[3 * n + d] - Ad[3 * n + d]) * l->BI[3 * n + d];
				/* scatter to self and lower neighbours through the transposed blocks */
				for(q = 0; q < 14; q++)
				{
					const int m = In[q];
					const double *b = Hn + 9 * q;
					if(m < 0)
						break;
					for(d = 0; d < 3; d++)
						Ad[3 * m + d] += b[d] * t[0] + b[3 + d] * t[1] + b[6 + d] * t[2];
				}
				for(d = 0; d < 3; d++)
					d0[3 * n + d] += t[d];
			}
		}
		else
		{
			int col;
			for(col = 0; col < 8; col++)
			{
				int x, y, z, d;
				for(y = (col >> 2) & 1; y < l->noy; y += 2)
					for(x = (col >> 1) & 1; x < l->nox; x += 2)
						for(z = col & 1; z < l->noz; z += 2)
						{
							int n = nidx(l, x, y, z);
							double r[3];
							row_mul(l, n, d0, r);
							for(d = 0; d < 3; d++)
								d0[3 * n + d] += (F[3 * n + d] - r[d]) * l->BI[3 * n + d];
						}
			}
		}
	}
	if(o->p.gs_colored)
		oracle_kmul(o, lev, d0, Ad, 1);
}

/* project_vector (Solver_multigrid.c:72-159): for every coarse element and
 * corner, the sum of the 8 nodal values of the fine sub-element at that
 * corner, weighted by TWW (= |J|), accumulated at the coarse node and scaled
 * by MASS (1 / lumped mass) */
void oracle_project_vector(oracle *o, int fine_lev, const double *AU, double *AD)
{
	const level *F = &o->lv[fine_lev], *C = &o->lv[fine_lev - 1];
	int e, a, j, d, n[8], cn[8];
	for(a = 0; a <= C->neq; a++)
		AD[a] = 0.0;
	for(e = 0; e < C->nel; e++)
	{
		int ez = e % C->elz, ex = (e / C->elz) % C->elx, ey = e / (C->elz * C->elx);
		elem_nodes(C, e, cn);
		for(a = 0; a < 8; a++)
		{
			int fe = eidx(F, 2 * ex + LOC[a][0], 2 * ey + LOC[a][1], 2 * ez + LOC[a][2]);
			double s[3] = {0.0, 0.0, 0.0};
			elem_nodes(F, fe, n);
			for(j = 0; j < 8; j++)
				for(d = 0; d < 3; d++)
					s[d] += AU[3 * n[j] + d];
			for(d = 0; d < 3; d++)
				AD[3 * cn[a] + d] += C->J * s[d];
		}
	}
	for(a = 0; a < C->nno; a++)
		for(d = 0; d < 3; d++)
			AD[3 * a + d] *= C->mass[a];
}

/* interp_vector (Solver_multigrid.c:173-298) with un_inject_vector (:581-624):
 * inject coincident nodes, then linear fill along x, z and y in that order
 * (uniform grid: weights 1/2, 1/2) */
void oracle_interp_vector(oracle *o, int coarse_lev, const double *AD, double *AU)
{
	const level *C = &o->lv[coarse_lev], *F = &o->lv[coarse_lev + 1];
	int x, y, z, d;
	for(x = 1; x <= F->neq; x++)
		AU[x] = 0.0;
	for(y = 0; y < C->noy; y++)
		for(x = 0; x < C->nox; x++)
			for(z = 0; z < C->noz; z++)
				for(d = 0; d < 3; d++)
					AU[3 * nidx(F, 2 * x, 2 * y, 2 * z) + d] = AD[3 * nidx(C, x, y, z) + d];
	for(y = 0; y < F->noy; y += 2)
		for(z = 0; z < F->noz; z += 2)
			for(x = 1; x < F->nox - 1; x += 2)
				for(d = 0; d < 3; d++)
					AU[3 * nidx(F, x, y, z) + d] = 0.5 * AU[3 * nidx(F, x - 1, y, z) + d] + 0.5 * AU[3 * nidx(F, x + 1, y, z) + d];
	for(y = 0; y < F->noy; y += 2)
		for(x = 0; x < F->nox; x++)
			for(z = 1; z < F->noz - 1; z += 2)
				for(d = 0; d < 3; d++)
					AU[3 * nidx(F, x, y, z) + d] = 0.5 * AU[3 * nidx(F, x, y, z - 1) + d] + 0.5 * AU[3 * nidx(F, x, y, z + 1) + d];
	for(x = 0; x < F->nox; x++)
		for(z = 0; z < F->noz; z++)
			for(y = 1; y < F->noy - 1; y += 2)
				for(d = 0; d < 3; d++)
					AU[3 * nidx(F, x, y, z) + d] = 0.5 * AU[3 * nidx(F, x, y - 1, z) + d] + 0.5 * AU[3 * nidx(F, x, y + 1, z) + d];
}

/* assemble_div_u (Element_calculations.c:691-722) */
void oracle_div_u(oracle *o, int lev, const double *U, double *divU)
{
	const level *l = &o->lv[lev];
	int e, a, d, n[8];
	for(e = 0; e < l->nel; e++)
	{
		double s = 0.0;
		elem_nodes(l, e, n);
		for(a = 0; a < 8; a++)
			for(d = 0; d < 3; d++)
				s += l->g[3 * a + d] * U[3 * n[a] + d];
		divU[e] = s;
	}
}

/* assemble_grad_p (Element_calculations.c:727-769) */
void oracle_grad_p(oracle *o, int lev, const double *P, double *gradP)
{
	const level *l = &o->lv[lev];
	int e, a, d, n[8];
	for(a = 0; a <= l->neq; a++)
		gradP[a] = 0.0;
	for(e = 0; e < l->nel; e++)
	{
		if(P[e] == 0.0)
			continue;
		elem_nodes(l, e, n);
		for(a = 0; a < 8; a++)
			for(d = 0; d < 3; d++)
				gradP[3 * n[a] + d] += l->g[3 * a + d] * P[e];
	}
	oracle_strip_bcs(o, lev, gradP);
}

static double vdot(int n, const double *a, const double *b)
{
	double s = 0.0;
	int i;
	for(i = 0; i < n; i++)
		s += a[i] * b[i];
	return s;
}

/* --------------------------------------------------------------- solvers */

/* multi_grid (General_matrix_functions.c:525-653) */
double oracle_multi_grid(oracle *o, double *d1, double *F, double acc)
{
	const int lmax = o->L - 1, lmin = 0;
	int lev, dlev, ulev, i, Vn;
	(void)acc;
	for(i = 0; i < o->lv[lmax].neq; i++)
		o->fl[lmax][i] = F[i];
	for(lev = lmax; lev > lmin; lev--)
	{
		oracle_project_vector(o, lev, o->fl[lev], o->fl[lev - 1]);
		oracle_strip_bcs(o, lev - 1, o->fl[lev - 1]);
	}
	oracle_gauss_seidel(o, lmin, o->vel[lmin], o->fl[lmin], o->AU[lmin], o->p.vlowstep, 0);
	for(lev = lmin + 1; lev <= lmax; lev++)
	{
		oracle_interp_vector(o, lev - 1, o->vel[lev - 1], o->vel[lev]);
		oracle_strip_bcs(o, lev, o->vel[lev]);
		for(i = 0; i < o->lv[lev].neq; i++)
			o->rhs[lev][i] = o->fl[lev][i];
		for(Vn = 1; Vn <= o->p.mg_cycle; Vn++)
		{
			for(dlev = lev; dlev >= lmin + 1; dlev--)
			{
				int cyc = (dlev == lmax) ? o->p.vhighstep : o->p.down_heavy;
				oracle_gauss_seidel(o, dlev, o->vel[dlev], o->rhs[dlev], o->AU[dlev], cyc, dlev == lev);
				for(i = 0; i < o->lv[dlev].neq; i++)
					o->res[dlev][i] = o->rhs[dlev][i] - o->AU[dlev][i];
				oracle_project_vector(o, dlev, o->res[dlev], o->rhs[dlev - 1]);
				oracle_strip_bcs(o, dlev - 1, o->rhs[dlev - 1]);
			}
			oracle_gauss_seidel(o, lmin, o->vel[lmin], o->rhs[lmin], o->AU[lmin], o->p.vlowstep, 0);
			for(ulev = lmin + 1; ulev <= lev; ulev++)
			{
				int cyc = (ulev == lmax) ? o->p.vhighstep : o->p.up_heavy;
				const int n = o->lv[ulev].neq;
				double audotau, alpha;
				oracle_interp_vector(o, ulev - 1, o->vel[ulev - 1], o->del_vel[ulev]);
				oracle_strip_bcs(o, ulev, o->del_vel[ulev]);
				oracle_gauss_seidel(o, ulev, o->del_vel[ulev], o->res[ulev], o->AU[ulev], cyc, 1);
				audotau = vdot(n, o->AU[ulev], o->AU[ulev]);
				alpha = vdot(n, o->AU[ulev], o->res[ulev]) / audotau;
				for(i = 0; i < n; i++)
					o->vel[ulev][i] += alpha * o->del_vel[ulev][i];
				if(ulev == lmax)
					for(i = 0; i < n; i++)
						o->res[ulev][i] -= alpha * o->AU[ulev][i];
			}
		}
	}
	for(i = 0; i < o->lv[lmax].neq; i++)
	{
		F[i] = o->res[lmax][i];
		d1[i] = o->vel[lmax][i];
	}
	return sqrt(vdot(o->lv[lmax].neq, F, F) / o->lv[lmax].neq);
}

/* solve_del2_u (General_matrix_functions.c:368-520), multigrid branch */
int oracle_solve_del2_u(oracle *o, double *d0, double *F, double acc, int *mg_calls)
{
	const int neq = o->lv[o->L - 1].neq;
	double residual, r0;
	int i, valid, count = 0;
	for(i = 0; i < neq; i++)
	{
		o->sr[i] = F[i];
		o->sAu[i] = d0[i] = o->sD1[i] = 0.0;
	}
	r0 = residual = sqrt(vdot(neq, o->sr, o->sr) / neq);
	if(r0 * o->p.accuracy > acc)
		acc = r0 * o->p.accuracy;
	valid = (residual < acc) ? 0 : 1;
	while(residual > acc)
	{
		residual = oracle_multi_grid(o, o->sD1, o->sr, acc);
		for(i = 0; i < neq; i++)
		{
			d0[i] += o->sD1[i];
			o->sD1[i] = 0.0;
		}
		count++;
	}
	if(mg_calls)
		*mg_calls += count;
	return valid;
}

/* The head of solve_Ahat_p_fhat (Stokes_flow_Incomp.c:360-371): V += K^-1
 * (F - G P - K V) solved to acc, then r1 = B V; returns |r1| / sqrt(npno). */
static double uzawa_head(oracle *o, double *V, const double *P, const double *F, double acc, double *r1, int *del2_calls,
                         int *mg_calls)
{
	const level *f = &o->lv[o->L - 1];
	const int npno = f->nel, neq = f->neq, lev = o->L - 1;
	double *Ah = o->Ah, *u1 = o->u1;
	int i;
	oracle_grad_p(o, lev, P, Ah);
	oracle_kmul(o, lev, V, u1, 1);
	for(i = 0; i < neq; i++)
		Ah[i] = F[i] - Ah[i] - u1[i];
	oracle_strip_bcs(o, lev, Ah);
	oracle_solve_del2_u(o, u1, Ah, acc, mg_calls);
	if(del2_calls)
		(*del2_calls)++;
	oracle_strip_bcs(o, lev, u1);
	for(i = 0; i < neq; i++)
		V[i] += u1[i];
	oracle_div_u(o, lev, V, r1);
	return sqrt(vdot(npno, r1, r1) / npno);
}

/* continuity residual of the residual rule: |B V| / (|V| sqrt(npno/neq)) */
static double continuity(double bvbv, double vv, int neq, int npno)
{
	return sqrt(bvbv / (vv > 0.0 ? vv : 1e-300) * ((double)neq / (double)npno));
}

/* solve_Ahat_p_fhat (Stokes_flow_Incomp.c:295-497); returns the initial
 * pressure residual as the reference does.  stop_rule 0 is the reference's
 * loop (dv/v and dp/p, :393, 442-443).  stop_rule 1 is the GPU library's
 * residual rule (no counterpart in the reference), restated step for step:
 * before every iteration the continuity residual of the recursively updated
 * r1 = B V is tested; once it is at most imp the momentum residual
 * |F - K V - G P| / |F| is evaluated, and above imp a velocity correction
 * (the head again, solved to imp/2 relative to |F|) follows and the search
 * direction restarts; at most 8 corrections. */
double oracle_solve_Ahat_p_fhat(oracle *o, double *V, double *P, const double *F, double imp, int *steps, int *del2_calls, int *mg_calls)
{
	const level *f = &o->lv[o->L - 1];
	const int npno = f->nel, neq = f->neq, lev = o->L - 1;
	const int gneq = neq;
	const int resid_rule = o->p.stop_rule == 1;
	double v_res, ff, residual, alpha, delta, s2dotAhat, r0dotr0, r1dotz1;
	double vdotv, pdotp, cont = 0.0;
	double dpressure = 1.0, dvelocity = 1.0;
	double *r0 = o->r0, *r1 = o->r1, *r2 = o->r2, *z0 = o->z0, *z1 = o->z1, *s1 = o->s1, *s2 = o->s2, *sh;
	double *Ah = o->Ah, *u1 = o->u1;
	int i, j, count = 0, valid, restart = 1;

	ff = vdot(neq, F, F);
	v_res = sqrt(ff / gneq);
	o->last_momentum = o->last_continuity = 0.0;
	o->last_corrections = 0;
	residual = uzawa_head(o, V, P, F, imp * v_res, r1, del2_calls, mg_calls);
	if(resid_rule)
		cont = continuity(residual * residual * npno, vdot(neq, V, V), neq, npno);

	for(;;)
	{
		if(resid_rule)
		{
			if(cont <= imp)
			{
				double rr = 0.0, mom, rc;
				oracle_grad_p(o, lev, P, Ah);
				oracle_kmul(o, lev, V, u1, 1);
				for(i = 0; i < neq; i++)
				{
					const double r = F[i] - Ah[i] - u1[i];
					rr += r * r;
				}
				mom = sqrt(rr / (ff > 0.0 ? ff : 1.0));
				o->last_momentum = mom;
				o->last_continuity = cont;
				if(mom <= imp || o->last_corrections >= 8)
					break;
				rc = uzawa_head(o, V, P, F, 0.5 * imp * v_res, r1, del2_calls, mg_calls);
				o->last_corrections++;
				cont = continuity(rc * rc * npno, vdot(neq, V, V), neq, npno);
				o->last_continuity = cont;
				restart = 1;
				continue;
			}
			if(count >= *steps)
				break;
		}
		else if(!((count < *steps) && (dpressure >= imp || dvelocity >= imp)))
			break;
		for(j = 0; j < npno; j++)
			z1[j] = f->BPI[j] * r1[j];
		r1dotz1 = vdot(npno, r1, z1);
		if(restart)
			for(j = 0; j < npno; j++)
				s2[j] = z1[j];
		else
		{
			r0dotr0 = vdot(npno, r0, z0);
			delta = r1dotz1 / r0dotr0;
			for(j = 0; j < npno; j++)
				s2[j] = z1[j] + delta * s1[j];
		}
		restart = 0;
		oracle_grad_p(o, lev, s2, Ah);
		valid = oracle_solve_del2_u(o, u1, Ah, imp * v_res, mg_calls);
		if(del2_calls)
			(*del2_calls)++;
		oracle_strip_bcs(o, lev, u1);
		oracle_div_u(o, lev, u1, Ah);
		s2dotAhat = vdot(npno, s2, Ah);
		alpha = valid ? r1dotz1 / s2dotAhat : 0.0;
		for(j = 0; j < npno; j++)
		{
			r2[j] = r1[j] - alpha * Ah[j];
			P[j] += alpha * s2[j];
		}
		for(j = 0; j < neq; j++)
			V[j] -= alpha * u1[j];
		oracle_div_u(o, lev, V, Ah);
		vdotv = vdot(neq, V, V);
		pdotp = vdot(npno, P, P);
		dpressure = alpha * sqrt(vdot(npno, s2, s2) / (1.0e-32 + pdotp));
		dvelocity = alpha * sqrt(vdot(neq, u1, u1) / (1.0e-32 + vdotv));
		if(resid_rule)
			cont = continuity(vdot(npno, r2, r2), vdotv, neq, npno);
		count++;
		sh = s1; s1 = s2; s2 = sh;
		sh = r0; r0 = r1; r1 = r2; r2 = sh;
		sh = z0; z0 = z1; z1 = sh;
	}
	/* the pointer rotation above permutes the work buffers; keep them owned */
	o->r0 = r0; o->r1 = r1; o->r2 = r2; o->z0 = z0; o->z1 = z1; o->s1 = s1; o->s2 = s2;
	*steps = count;
	return residual;
}

void oracle_last_residuals(const oracle *o, double out[3])
{
	out[0] = o->last_momentum;
	out[1] = o->last_continuity;
	out[2] = o->last_corrections;
}

/* general_stokes_solver (Drive_solvers.c:45-165), with
 * construct_stiffness_B_matrix (Construct_arrays.c:834-889) and
 * solve_constrained_flow_iterative / v_from_vector (Stokes_flow_Incomp.c:50-90,
 * 530-553).  With SDEPV the viscosity, operator and solve repeat
 * (:120-159): after each solve U <- a U + (1 - a) oldU (damping a =
 * sdepv_iter_damp, when it is not 1), then |U - oldU| / |U| is the misfit and
 * oldU <- U, until the misfit is at most sdepv_misfit or max_sdep_visc_iter
 * solves ran.  *steps, *del2_calls and *mg_calls add up over the solves. */
double oracle_stokes(oracle *o, int *steps, int *del2_calls, int *mg_calls)
{
	const level *f = &o->lv[o->L - 1];
	const int iterate = o->p.sdepv != 0;
	double r = 0.0, misfit = 0.0;
	int n, d, i, count = 0, total_steps = 0, total_del2 = 0, total_mg = 0;
	for(n = 0; n < f->nno; n++)
		for(d = 0; d < 3; d++)
			if(f->vflag[n] & (1u << d))
				o->U[3 * n + d] = 0.0;
	oracle_assemble_forces(o);
	do
	{
		int st = o->p.piterations, dc = 0, mc = 0;
		if(o->p.tdepv || o->p.sdepv)
			oracle_get_system_viscosity(o);
		oracle_project_viscosity(o);
		oracle_construct_stiffness(o);
		r = oracle_solve_Ahat_p_fhat(o, o->U, o->P, o->F, o->p.accuracy, &st, &dc, &mc);
		total_steps += st;
		total_del2 += dc;
		total_mg += mc;
		for(n = 0; n < f->nno; n++)
			for(d = 0; d < 3; d++)
				o->V[d][n] = (f->vflag[n] & (1u << d)) ? 0.0 : o->U[3 * n + d];
		count++;
		if(iterate)
		{
			const double a = o->p.sdepv_iter_damp;
			double uu = 0.0, dd = 0.0;
			for(i = 0; i < f->neq; i++)
			{
				if(fabs(a - 1.0) > 1e-7)
					o->U[i] = a * o->U[i] + (1.0 - a) * o->oldU[i];
				const double du = o->U[i] - o->oldU[i];
				o->oldU[i] = o->U[i];
				uu += o->U[i] * o->U[i];
				dd += du * du;
			}
			misfit = uu != 0.0 ? sqrt(dd) / sqrt(uu) : sqrt(dd);
		}
	} while(iterate && misfit > o->p.sdepv_misfit && count < o->p.max_sdep_visc_iter);
	*steps = total_steps;
	*del2_calls = total_del2;
	*mg_calls = total_mg;
	return r;
}

/* ---------------------------------------------------------------- energy */

/* std_timestep (Advection_diffusion.c:737-810) */
static void std_timestep(oracle *o)
{
	const level *f = &o->lv[o->L - 1];
	double diff_ts, adv_ts = 1.0e8;
	int e, a, d, n[8];
	if(o->p.fixed_timestep != 0.0)
	{
		o->timestep = o->p.fixed_timestep;
		return;
	}
	diff_ts = 1.0e8;
	for(d = 0; d < 3; d++)
		if(f->h[d] * f->h[d] < diff_ts)
			diff_ts = f->h[d] * f->h[d];
	diff_ts *= 0.5;
	for(e = 0; e < f->nel; e++)
	{
		double uc[3] = {0, 0, 0}, u;
		elem_nodes(f, e, n);
		for(a = 0; a < 8; a++)
			for(d = 0; d < 3; d++)
				uc[d] += 0.125 * o->V[d][n[a]];
		u = fabs(uc[0]) / f->h[0] + fabs(uc[1]) / f->h[1] + fabs(uc[2]) / f->h[2];
		if(0.5 / u < adv_ts)
			adv_ts = 0.5 / u;
	}
	adv_ts = o->p.finetunedt * adv_ts;
	o->timestep = 1.0e-32 + (adv_ts < diff_ts ? adv_ts : diff_ts);
}

/* pg_solver (Advection_diffusion.c:398-440) with pg_shape_fn (:448-555) and
 * element_residual (:564-727), Cartesian, diffusivity 1, Q = Q0, no flux BC */
static void pg_solver(oracle *o, double *DTdot)
{
	const level *f = &o->lv[o->L - 1];
	const double diff = 1.0, twodiff = 2.0 * diff;
	int e, a, k, d, n[8];
	for(a = 0; a < f->nno; a++)
		DTdot[a] = 0.0;
	for(e = 0; e < f->nel; e++)
	{
		double uc[3] = {0, 0, 0}, us[3], up[3], adiff, unorm;
		double PG[8][8], v[8][3], tx[8][3], dT[8], Eres[8];
		elem_nodes(f, e, n);
		for(a = 0; a < 8; a++)
			for(d = 0; d < 3; d++)
				uc[d] += 0.125 * o->V[d][n[a]];
		for(d = 0; d < 3; d++)
		{
			us[d] = fabs(uc[d] * f->h[d]);
			up[d] = (us[d] > twodiff) ? (1.0 - twodiff / us[d]) : 0.0;
		}
		unorm = uc[0] * uc[0] + uc[1] * uc[1] + uc[2] * uc[2];
		adiff = (unorm > 0.000001) ? ((us[0] * up[0] + us[1] * up[1] + us[2] * up[2]) / (2.0 * unorm)) : 0.0;
		for(k = 0; k < 8; k++)
		{
			for(d = 0; d < 3; d++)
			{
				v[k][d] = 0.0;
				tx[k][d] = 0.0;
			}
			dT[k] = 0.0;
			for(a = 0; a < 8; a++)
			{
				double DT = o->tflag[n[a]] ? 0.0 : o->Tdot[n[a]];
				dT[k] += DT * o->Nv[k][a];
				for(d = 0; d < 3; d++)
				{
					v[k][d] += o->V[d][n[a]] * o->Nv[k][a];
					tx[k][d] += f->gnx[k][a][d] * o->T[n[a]];
				}
			}
			for(a = 0; a < 8; a++)
				PG[k][a] = o->Nv[k][a] + adiff * (v[k][0] * f->gnx[k][a][0] + v[k][1] * f->gnx[k][a][1] + v[k][2] * f->gnx[k][a][2]);
		}
		for(a = 0; a < 8; a++)
		{
			Eres[a] = 0.0;
			for(k = 0; k < 8; k++)
				Eres[a] -= PG[k][a] * f->J * (dT[k] - o->p.Q0 + v[k][0] * tx[k][0] + v[k][1] * tx[k][1] + v[k][2] * tx[k][2]) +
					diff * f->J * (f->gnx[k][a][0] * tx[k][0] + f->gnx[k][a][1] * tx[k][1] + f->gnx[k][a][2] * tx[k][2]);
			DTdot[n[a]] += Eres[a];
		}
	}
	for(a = 0; a < f->nno; a++)
		DTdot[a] *= f->mass[a];
}

static double tmax(const oracle *o)
{
	const level *f = &o->lv[o->L - 1];
	double t = -10.0;
	int n;
	for(n = 0; n < f->nno; n++)
		if(o->T[n] > t)
			t = o->T[n];
	return t;
}

/* PG_timestep (Advection_diffusion.c:251-345) with predictor/corrector
 * (:352-386), temperatures_conform_bcs (Boundary_conditions.c:949-991) and
 * thermal_buoyancy */
void oracle_pg_timestep(oracle *o)
{
	const level *f = &o->lv[o->L - 1];
	const double gamma = 0.5;
	double *DTdot = (double *)xcalloc(f->nno, sizeof(double));
	double *T1 = (double *)xcalloc(f->nno, sizeof(double));
	double *Tdot1 = (double *)xcalloc(f->nno, sizeof(double));
	double T_interior1, dt_reduced = 1.0;
	int n, iredo, sub = 1, pass;

	std_timestep(o);
	for(n = 0; n < f->nno; n++)
	{
		T1[n] = o->T[n];
		Tdot1[n] = o->Tdot[n];
	}
	T_interior1 = tmax(o);
	do
	{
		o->timestep *= dt_reduced;
		iredo = 0;
		for(n = 0; n < f->nno; n++)
		{
			if(!o->tflag[n])
				o->T[n] += (1.0 - gamma) * o->timestep * o->Tdot[n];
			o->Tdot[n] = 0.0;
		}
		for(pass = 0; pass < o->p.adv_sub_iterations; pass++)
		{
			pg_solver(o, DTdot);
			for(n = 0; n < f->nno; n++)
			{
				if(!o->tflag[n])
					o->T[n] += gamma * o->timestep * DTdot[n];
				o->Tdot[n] += DTdot[n];
			}
		}
		o->T_interior = tmax(o);
		if(o->T_interior / T_interior1 > 1.01)
		{
			for(n = 0; n < f->nno; n++)
			{
				o->T[n] = T1[n];
				o->Tdot[n] = Tdot1[n];
			}
			iredo = 1;
			dt_reduced *= 0.5;
			sub++;
		}
	} while(iredo == 1 && sub <= 5);
	o->elapsed += o->timestep;
	for(n = 0; n < f->nno; n++)
		if(o->tflag[n])
			o->T[n] = ((n % f->noz) == 0) ? 1.0 : 0.0;
	oracle_thermal_buoyancy(o);
	free(DTdot);
	free(T1);
	free(Tdot1);
}

/* heat_flux (Process_buoyancy.c:63-203): nodal vertical heat flux, surface
 * extrapolation and the area-weighted surface means Nut / Nub */
void oracle_heat_flux(oracle *o, double *nut, double *nub)
{
	const level *f = &o->lv[o->L - 1];
	const double diff = 1.0;
	double *hf = (double *)xcalloc(f->nno, sizeof(double));
	double *sh, *bh;
	double hft = 0, hfb = 0, areat = 0, areab = 0;
	int e, k, a, n[8], x, y;
	for(e = 0; e < f->nel; e++)
	{
		double uT = 0.0;
		elem_nodes(f, e, n);
		for(k = 0; k < 8; k++)
		{
			double u = 0, T = 0, dTdz = 0;
			for(a = 0; a < 8; a++)
			{
				u += o->V[2][n[a]] * o->Nv[k][a];
				T += o->T[n[a]] * o->Nv[k][a];
				dTdz += o->T[n[a]] * f->gnx[k][a][2];
			}
			uT += (u * T - diff * dTdz) * f->J;
		}
		uT /= 8.0 * f->J;
		for(a = 0; a < 8; a++)
			hf[n[a]] += f->J * uT;
	}
	for(a = 0; a < f->nno; a++)
		hf[a] *= f->mass[a];
	sh = (double *)xcalloc((size_t)f->nox * f->noy, sizeof(double));
	bh = (double *)xcalloc((size_t)f->nox * f->noy, sizeof(double));
	for(y = 0; y < f->noy; y++)
		for(x = 0; x < f->nox; x++)
		{
			int top = nidx(f, x, y, f->noz - 1), bot = nidx(f, x, y, 0);
			sh[x + y * f->nox] = 2.0 * hf[top] - hf[top - 1];
			bh[x + y * f->nox] = 2.0 * hf[bot] - hf[bot + 1];
		}
	for(y = 0; y < f->ely; y++)
		for(x = 0; x < f->elx; x++)
		{
			double area = 8.0 * f->J;
			double tt = sh[x + y * f->nox] + sh[x + 1 + y * f->nox] + sh[x + 1 + (y + 1) * f->nox] + sh[x + (y + 1) * f->nox];
			double tb = bh[x + y * f->nox] + bh[x + 1 + y * f->nox] + bh[x + 1 + (y + 1) * f->nox] + bh[x + (y + 1) * f->nox];
			hft += tt * area;
			hfb += tb * area;
			areat += area;
			areab += area;
		}
	*nut = hft / (areat * 4.0);
	*nub = hfb / (areab * 4.0);
	free(hf);
	free(sh);
	free(bh);
}

/* Vrms = sqrt(int |u|^2 dV / V), 2x2x2 Gauss over the Q1 elements.  The
 * reference writes only a depth profile (Process_velocity.c:200-214); this
 * scalar is the project's definition, applied identically to every code. */
double oracle_vrms(oracle *o)
{
	const level *f = &o->lv[o->L - 1];
	double s = 0.0, vol = 0.0;
	int e, k, a, n[8];
	for(e = 0; e < f->nel; e++)
	{
		elem_nodes(f, e, n);
		for(k = 0; k < 8; k++)
		{
			double u[3] = {0, 0, 0};
			int d;
			for(a = 0; a < 8; a++)
				for(d = 0; d < 3; d++)
					u[d] += o->Nv[k][a] * o->V[d][n[a]];
			s += f->J * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
			vol += f->J;
		}
	}
	return sqrt(s / vol);
}
