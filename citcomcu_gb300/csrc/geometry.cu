// Element geometry of the regional spherical shell segment (Geometry=Rsphere),
// host side: one Geo entry per (theta, r) column of elements of a level.
//
// Nodes sit on a uniform grid in (theta, phi, r) (Nodal_mesh.c:87-95,
// 202-217); velocity components are the local spherical ones (u_theta, u_phi,
// u_r) of each node.  Every element of a column is the element of phi index 0
// rotated about the polar axis, and every quantity below is a scalar or a
// component in local spherical frames, so it is the same for the whole
// column.  Restated from:
//   get_global_shape_fn, spherical branch (Size_does_matter.c:60-179): |J|
//     and the global shape-function derivatives, rotated by form_rtf_bc
//     (:182-200) into d/dtheta, d/dphi, d/dr;
//   get_rtf (:203-251): theta and 1/r at the Gauss points;
//   construct_c3x3matrix_el (:253-445): dot products of the node frames with
//     the Gauss-point frame and with its theta / phi derivatives;
//   get_ba, spherical branch (Element_calculations.c:300-350) and the
//     Rsphere strain-rate form of get_elt_k (:249-259);
//   get_elt_g, Rsphere branch (:899-925), one pressure point of weight 8;
//   mass_matrix (Size_does_matter.c:618-757): TWW, element volume, sizes.
#include <cmath>
#include <cstring>

#include "kernels.h"

namespace {

constexpr double BETA = 0.57735026918962576451;

inline double sgn(int a, int d) { return cg_loc(a, d) ? 1.0 : -1.0; }

// trilinear shape function of local node a and its xi_d derivative
double shp(int a, const double xi[3])
{
	double v = 1.0;
	for(int d = 0; d < 3; ++d)
		v *= 0.5 * (1.0 + sgn(a, d) * xi[d]);
	return v;
}

double dshp(int a, int d, const double xi[3])
{
	double v = 0.5 * sgn(a, d);
	for(int e = 0; e < 3; ++e)
		if(e != d)
			v *= 0.5 * (1.0 + sgn(a, e) * xi[e]);
	return v;
}

double det3(const double A[3][3])
{
	return A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
	       A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
}

double myatan(double y, double x)
{
	double f = atan2(y, x);
	return f < 0.0 ? f + 2.0 * M_PI : f;
}

// local spherical frame at (theta, phi): rows e_theta, e_phi, e_r
void frame(double t, double f, double u[3][3])
{
	const double ct = cos(t), cf = cos(f), st = sin(t), sf = sin(f);
	u[0][0] = ct * cf;
	u[0][1] = ct * sf;
	u[0][2] = -st;
	u[1][0] = -sf;
	u[1][1] = cf;
	u[1][2] = 0.0;
	u[2][0] = st * cf;
	u[2][1] = st * sf;
	u[2][2] = ct;
}

// Geometry at one reference point xi of an element with Cartesian node
// coordinates X and spherical node angles SA (theta, phi)
struct Point
{
	double gnx[8][3];   // d/dtheta, d/dphi, d/dr of N_a
	double jac;         // |J|
	double theta, rinv;
	double cc[3][3][8];     // [gauss frame g][node frame n][a]
	double ccx[3][3][2][8]; // [g][n][d = theta, phi][a]
};

void point(const double X[8][3], const double SA[8][2], const double xi[3], Point &P)
{
	// dxda[d][e] = sum_i X_e(i) dN_i/dxi_d
	double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
	for(int i = 0; i < 8; ++i)
		for(int d = 0; d < 3; ++d)
		{
			const double dn = dshp(i, d, xi);
			for(int e = 0; e < 3; ++e)
				A[d][e] += X[i][e] * dn;
		}
	P.jac = det3(A);
	// cofactors: cof[e][d]; Cartesian derivative dN/dx_d = sum_e dN/dxi_e cof[e][d] / |J|
	double cof[3][3];
	for(int r = 0; r < 3; ++r)
		for(int c = 0; c < 3; ++c)
		{
			const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
			cof[r][c] = A[r1][c1] * A[r2][c2] - A[r1][c2] * A[r2][c1];
		}
	double gc[8][3];
	for(int j = 0; j < 8; ++j)
		for(int d = 0; d < 3; ++d)
		{
			double v = 0.0;
			for(int e = 0; e < 3; ++e)
				v += dshp(j, e, xi) * cof[e][d];
			gc[j][d] = v / P.jac;
		}
	// position of the point, its theta, phi, 1/r and the rotation form_rtf_bc
	double x[3] = {0, 0, 0};
	for(int i = 0; i < 8; ++i)
	{
		const double n = shp(i, xi);
		for(int e = 0; e < 3; ++e)
			x[e] += X[i][e] * n;
	}
	P.rinv = 1.0 / sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
	P.theta = acos(x[2] * P.rinv);
	const double phi = myatan(x[1], x[0]);
	const double bc[3][3] = {{x[2] * cos(phi), x[2] * sin(phi), -sin(P.theta) / P.rinv}, {-x[1], x[0], 0.0},
	                         {x[0] * P.rinv, x[1] * P.rinv, x[2] * P.rinv}};
	for(int j = 0; j < 8; ++j)
		for(int d = 0; d < 3; ++d)
			P.gnx[j][d] = bc[d][0] * gc[j][0] + bc[d][1] * gc[j][1] + bc[d][2] * gc[j][2];
	// frames: Gauss point (and its theta / phi derivatives) against each node's
	double u[3][3], ux[2][3][3];
	frame(P.theta, phi, u);
	{
		const double ct = cos(P.theta), cf = cos(phi), st = sin(P.theta), sf = sin(phi);
		const double d_t[3][3] = {{-st * cf, -st * sf, -ct}, {0.0, 0.0, 0.0}, {ct * cf, ct * sf, -st}};
		const double d_f[3][3] = {{-ct * sf, ct * cf, 0.0}, {-cf, -sf, 0.0}, {-st * sf, st * cf, 0.0}};
		memcpy(ux[0], d_t, sizeof(d_t));
		memcpy(ux[1], d_f, sizeof(d_f));
	}
	for(int a = 0; a < 8; ++a)
	{
		double ua[3][3];
		frame(SA[a][0], SA[a][1], ua);
		for(int g = 0; g < 3; ++g)
			for(int n = 0; n < 3; ++n)
			{
				P.cc[g][n][a] = ua[n][0] * u[g][0] + ua[n][1] * u[g][1] + ua[n][2] * u[g][2];
				for(int d = 0; d < 2; ++d)
					P.ccx[g][n][d][a] = ua[n][0] * ux[d][g][0] + ua[n][1] * ux[d][g][1] + ua[n][2] * ux[d][g][2];
			}
	}
}

void fill_column(const Lvl &L, int ex, int ez, Geo *G)
{
	memset(G, 0, sizeof(Geo));
	double X[8][3], SA[8][2], R[8];
	for(int a = 0; a < 8; ++a)
	{
		const double t = L.org[0] + (ex + cg_loc(a, 0)) * L.h[0];
		const double f = L.org[1] + cg_loc(a, 1) * L.h[1];
		const double r = L.org[2] + (ez + cg_loc(a, 2)) * L.h[2];
		SA[a][0] = t;
		SA[a][1] = f;
		R[a] = r;
		X[a][0] = r * sin(t) * cos(f);
		X[a][1] = r * sin(t) * sin(f);
		X[a][2] = r * cos(t);
	}
	// Gauss points: the node sign pattern times BETA; weight 1
	double ba[8][3][8][6];  // [a][i][k][component] (get_ba)
	for(int k = 0; k < 8; ++k)
	{
		const double xi[3] = {sgn(k, 0) * BETA, sgn(k, 1) * BETA, sgn(k, 2) * BETA};
		Point P;
		point(X, SA, xi, P);
		G->gda[k] = P.jac;
		G->rinv[k] = P.rinv;
		G->rsin[k] = P.rinv / sin(P.theta);
		const double ra = P.rinv, si = 1.0 / sin(P.theta), ct = cos(P.theta) * si;
		for(int a = 0; a < 8; ++a)
		{
			const double sh = shp(a, xi);
			G->N[k][a] = sh;
			for(int d = 0; d < 3; ++d)
				G->gnx[k][a][d] = P.gnx[a][d];
			const double g0 = P.gnx[a][0], g1 = P.gnx[a][1], g2 = P.gnx[a][2];
			for(int i = 0; i < 3; ++i)
			{
				const double c1 = P.cc[0][i][a], c2 = P.cc[1][i][a], c3 = P.cc[2][i][a];
				G->cr[k][a][i] = c3;
				ba[a][i][k][0] = ((g0 * c1 + sh * P.ccx[0][i][0][a]) + sh * c3) * ra;
				ba[a][i][k][1] = (sh * c1 * ct + sh * c3 + (g1 * c2 + sh * P.ccx[1][i][1][a]) * si) * ra;
				ba[a][i][k][2] = g2 * c3;
				ba[a][i][k][3] = ((g0 * c2 + sh * P.ccx[1][i][0][a]) - sh * c2 * ct + (g1 * c1 + sh * P.ccx[0][i][1][a]) * si) * ra;
				ba[a][i][k][4] = g2 * c1 + (g0 * c3 + sh * (P.ccx[2][i][0][a] - c1)) * ra;
				ba[a][i][k][5] = g2 * c2 + ((g1 * c3 + sh * P.ccx[2][i][1][a]) * si - sh * c2) * ra;
			}
		}
	}
	for(int k = 0; k < 8; ++k)
		for(int a = 0; a < 8; ++a)
			for(int b = 0; b < 8; ++b)
				for(int i = 0; i < 3; ++i)
					for(int j = 0; j < 3; ++j)
					{
						const double *p = ba[a][i][k], *q = ba[b][j][k];
						G->Mk[k][a][b][3 * i + j] =
							G->gda[k] * (2.0 * (p[0] * q[0] + p[1] * q[1] + p[2] * q[2]) + p[3] * q[3] + p[4] * q[4] + p[5] * q[5]);
					}
	// the pressure point (element centre, weight 8): get_elt_g
	{
		const double xi[3] = {0.0, 0.0, 0.0};
		Point P;
		point(X, SA, xi, P);
		const double temp = 8.0 * P.jac;
		const double ra = P.rinv, si = 1.0 / sin(P.theta), ct = cos(P.theta) * si;
		G->rinvc = P.rinv;
		G->thetac = P.theta;
		for(int a = 0; a < 8; ++a)
			for(int d = 0; d < 3; ++d)
				G->gnxc[a][d] = P.gnx[a][d];
		for(int a = 0; a < 8; ++a)
		{
			const double n = shp(a, xi);
			for(int i = 0; i < 3; ++i)
			{
				const double x = P.gnx[a][2] * P.cc[2][i][a] + 2.0 * ra * n * P.cc[2][i][a] +
				                 ra * (P.gnx[a][0] * P.cc[0][i][a] + n * P.ccx[0][i][0][a] + ct * n * P.cc[0][i][a] +
				                       si * (P.gnx[a][1] * P.cc[1][i][a] + n * P.ccx[1][i][1][a]));
				G->g[3 * a + i] = -x * temp;
			}
		}
	}
	// mass_matrix: TWW = int N_a, volume, sizes from the centroid of the nodes
	for(int a = 0; a < 8; ++a)
	{
		double t = 0.0;
		for(int k = 0; k < 8; ++k)
			t += G->gda[k] * G->N[k][a];
		G->tww[a] = t;
	}
	for(int k = 0; k < 8; ++k)
		G->area += G->gda[k];
	double c[3] = {0, 0, 0};
	for(int a = 0; a < 8; ++a)
		for(int e = 0; e < 3; ++e)
			c[e] += X[a][e];
	for(int e = 0; e < 3; ++e)
		c[e] /= 8.0;
	const double rc = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]), tc = acos(c[2] / rc), fc = myatan(c[1], c[0]);
	// node order of the reference (1..4 the lower face): a = 0 (n1), 1 (n2), 2 (n3), 3 (n4)
	const double dt = fmax(fabs(SA[2][0] - SA[0][0]), fabs(SA[1][0] - SA[3][0]));
	const double df = fmax(fabs(SA[2][1] - SA[0][1]), fabs(SA[1][1] - SA[3][1]));
	const double dr = 0.25 * (R[4] + R[5] + R[6] + R[7] - R[0] - R[1] - R[2] - R[3]);
	G->size[0] = dt * rc;
	G->size[1] = df * rc * sin(tc);
	G->size[2] = fabs(dr);
	// get_global_1d_shape_fn, Rsphere branch (Size_does_matter.c:447-532): the
	// lower face's nodes in the tangent plane at the element centre; |J| of
	// that plane map at the face's 2x2 Gauss points, and each node's weight
	// int M_a dGamma (return_horiz_ave, Global_operations.c:133-251)
	{
		double u[3][3];
		frame(tc, fc, u);
		double xx[4][2];
		for(int i = 0; i < 4; ++i)
			for(int e = 0; e < 2; ++e)
				xx[i][e] = X[i][0] * u[e][0] + X[i][1] * u[e][1] + X[i][2] * u[e][2];
		for(int i = 0; i < 4; ++i)
			G->wface[i] = 0.0;
		for(int g = 0; g < 4; ++g)
		{
			const double xi = sgn(g, 0) * BETA, eta = sgn(g, 1) * BETA;
			double A[2][2] = {{0, 0}, {0, 0}};
			double M[4];
			for(int i = 0; i < 4; ++i)
			{
				const double sx = sgn(i, 0), sy = sgn(i, 1);
				M[i] = 0.25 * (1.0 + sx * xi) * (1.0 + sy * eta);
				const double d0 = 0.25 * sx * (1.0 + sy * eta), d1 = 0.25 * sy * (1.0 + sx * xi);
				for(int e = 0; e < 2; ++e)
				{
					A[0][e] += xx[i][e] * d0;
					A[1][e] += xx[i][e] * d1;
				}
			}
			const double jac = A[0][0] * A[1][1] - A[0][1] * A[1][0];
			for(int i = 0; i < 4; ++i)
				G->wface[i] += M[i] * jac;
		}
	}
}

} // namespace

void geo_fill_sphere(const Lvl &L, Geo *g)
{
	for(int ex = 0; ex < L.elx; ++ex)
		for(int ez = 0; ez < L.elz; ++ez)
			fill_column(L, ex, ez, g + cg_col(L, ex, ez));
}
