// Device helpers shared by the kernel translation units (included inside
// each unit's anonymous namespace).
#pragma once

#include <cuda_runtime.h>

#include "level.h"

// Programmatic dependent launch: every kernel first waits for its
// predecessor in the stream to finish (griddepcontrol.wait), then lets its own
// successor start launching (griddepcontrol.launch_dependents), so the launch
// latency of the next kernel overlaps this kernel's execution.  Both are
// no-ops when a kernel was launched without the attribute.
__device__ __forceinline__ void pdl_begin()
{
	asm volatile("griddepcontrol.wait;" ::: "memory");
	asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ int colour_of_pos(const Lvl &L, int p)
{
	int c = 0;
#pragma unroll
	for(int k = 1; k < 8; ++k)
		c += (p >= L.coff[k]);
	return c;
}

__device__ __forceinline__ void pos_xyz(const Lvl &L, int p, int &c, int &x, int &y, int &z)
{
	c = colour_of_pos(L, p);
	cg_decode(L, c, p - L.coff[c], x, y, z);
}

// Relaxation of small FP32 levels with the correction vector in shared
// memory on a grid with a one-node zero halo (the neighbour of every slot is
// then a fixed offset from the node and needs no clamping; stencil blocks of
// missing neighbours are zero).  Nine lanes serve one node: lane r9 =
// 3(dy+1) + (dx+1) takes the slots 3r9 .. 3r9+2 (dz = -1, 0, 1), whose
// neighbours are three consecutive halo cells, and the 27 stencil words of
// those slots (all three rows), padded to 28: "padded stencil" Kt, 252 words
// per node, Kt[252p + 28r9 + 9k + 3i + j] = K_ij of slot 3r9 + k.  The nine
// lanes of a node read 1008 consecutive bytes of stencil and 432 of vector.
constexpr int KT_WORDS = 252;

// rows r_i = sum over the lane's three slots of K_ij u_j
__device__ __forceinline__ void kt_rows(const float4 *kr, const float4 *ur, float &r0, float &r1, float &r2)
{
	float k[28];
#pragma unroll
	for(int q = 0; q < 7; ++q)
	{
		const float4 v = kr[q];
		k[4 * q] = v.x;
		k[4 * q + 1] = v.y;
		k[4 * q + 2] = v.z;
		k[4 * q + 3] = v.w;
	}
	r0 = r1 = r2 = 0.f;
#pragma unroll
	for(int kk = 0; kk < 3; ++kk)
	{
		const float4 u = ur[kk];
		r0 += k[9 * kk + 0] * u.x + k[9 * kk + 1] * u.y + k[9 * kk + 2] * u.z;
		r1 += k[9 * kk + 3] * u.x + k[9 * kk + 4] * u.y + k[9 * kk + 5] * u.z;
		r2 += k[9 * kk + 6] * u.x + k[9 * kk + 7] * u.y + k[9 * kk + 8] * u.z;
	}
}

// sum of a row value over the nine lanes 9*sub .. 9*sub+8 of a node; the
// total is valid in lane 9*sub (all 32 lanes must call it)
__device__ __forceinline__ float kt_sum9(float v, int lane)
{
	v += __shfl_sync(0xffffffffu, v, min(lane + 1, 31)) + __shfl_sync(0xffffffffu, v, min(lane + 2, 31));
	v += __shfl_sync(0xffffffffu, v, min(lane + 3, 31)) + __shfl_sync(0xffffffffu, v, min(lane + 6, 31));
	return v;
}


// loads of data that other CTAs of a cluster wrote earlier in the same
// kernel go to L2 (CG = true); plain loads otherwise
template <bool CG, typename T> __device__ __forceinline__ T ldv(const T *p)
{
	if constexpr(CG)
		return __ldcg(p);
	else
		return *p;
}

// project_vector (Solver_multigrid.c:72-159), node-centred: 8 consecutive
// lanes serve one coarse node, lane a its coarse element at corner a (the
// fine sub-element of that corner), weighted by that element's TWW of the
// node; the lanes' sums are added by shuffles and divided by the node's
// lumped mass (the sum of the weights).  Followed by strip_bcs_from_residual
// on the coarse level.  t is the lane's global index (coarse node t / 8); all
// 32 lanes of a warp must call it.  ACC: the type the sums are formed in.
template <bool CG, typename T, typename ACC = double>
__device__ __forceinline__ void project_lanes(const Lvl &Lf, const Lvl &Lc, const Geo *gc, const T *AU, T *AD, int t)
{
	const int N = t >> 3, a = t & 7;
	ACC s0 = 0, s1 = 0, s2 = 0, w = 0;
	int X = 0, Y = 0, Z = 0;
	if(N < Lc.nno)
	{
		Z = N % Lc.noz;
		X = (N / Lc.noz) % Lc.nox;
		Y = N / (Lc.noz * Lc.nox);
		const int ox = cg_loc(a, 0), oy = cg_loc(a, 1), oz = cg_loc(a, 2);
		const int ex = X - ox, ey = Y - oy, ez = Z - oz;
		if(ex >= 0 && ex < Lc.elx && ey >= 0 && ey < Lc.ely && ez >= 0 && ez < Lc.elz)
		{
			w = (ACC)gc[cg_col(Lc, ex, ez)].tww[a];
			const int fx = 2 * ex + ox, fy = 2 * ey + oy, fz = 2 * ez + oz;
			ACC t0 = 0, t1 = 0, t2 = 0;
#pragma unroll
			for(int b = 0; b < 8; ++b)
			{
				const int m = cg_node(Lf, fx + cg_loc(b, 0), fy + cg_loc(b, 1), fz + cg_loc(b, 2));
				t0 += (ACC)ldv<CG>(AU + 3 * m);
				t1 += (ACC)ldv<CG>(AU + 3 * m + 1);
				t2 += (ACC)ldv<CG>(AU + 3 * m + 2);
			}
			s0 = w * t0;
			s1 = w * t1;
			s2 = w * t2;
		}
	}
	// fixed-order sum over the 8 corners (lane a of the group holds corner a)
	for(int o = 1; o < 8; o <<= 1)
	{
		s0 += __shfl_xor_sync(0xffffffffu, s0, o);
		s1 += __shfl_xor_sync(0xffffffffu, s1, o);
		s2 += __shfl_xor_sync(0xffffffffu, s2, o);
		w += __shfl_xor_sync(0xffffffffu, w, o);
	}
	if(N < Lc.nno && a == 0)
	{
		const ACC mass = (ACC)1 / w;
		const unsigned f = cg_vflag(Lc, X, Y, Z);
		AD[3 * N] = (f & 1u) ? (T)0 : (T)(s0 * mass);
		AD[3 * N + 1] = (f & 2u) ? (T)0 : (T)(s1 * mass);
		AD[3 * N + 2] = (f & 4u) ? (T)0 : (T)(s2 * mass);
	}
}

// interp_vector (Solver_multigrid.c:173-298): injection, then linear fill
// along x (y,z even), along z (y even) and along y, in that order; evaluated
// per fine node with the same operation order.  Strips the fine level.  The
// fill weights are x2 / (x1 + x2), x1 / (x1 + x2) with x1, x2 the sizes (along
// the fill) of the first elements of the two neighbours (element index order:
// corner (max(X-1, 0), ., max(Z-1, 0))): 1/2 on the box; in the sphere the
// theta and r sizes of an element depend on its column.  SPH selects the
// spherical weights at compile time (the box variant then holds no geometry
// reads: 65 instead of 92 registers).
template <bool CG, typename T> __device__ __forceinline__ T coarse_at(const Lvl &Lc, const T *AD, int x, int y, int z, int d)
{
	return ldv<CG>(AD + 3 * cg_node(Lc, x >> 1, y >> 1, z >> 1) + d);
}
template <bool CG, bool SPH, typename T>
__device__ __forceinline__ T fill_x(const Lvl &Lc, const Lvl &Lf, const Geo *gf, const T *AD, int x, int y, int z, int d)
{
	if(x & 1)
	{
		if(SPH)
		{
			const int ez = z > 0 ? z - 1 : 0;
			const double x1 = gf[cg_col(Lf, x >= 2 ? x - 2 : 0, ez)].size[0], x2 = gf[cg_col(Lf, x, ez)].size[0];
			return (T)(x2 / (x1 + x2)) * coarse_at<CG>(Lc, AD, x - 1, y, z, d) +
			       (T)(x1 / (x1 + x2)) * coarse_at<CG>(Lc, AD, x + 1, y, z, d);
		}
		return (T)0.5 * coarse_at<CG>(Lc, AD, x - 1, y, z, d) + (T)0.5 * coarse_at<CG>(Lc, AD, x + 1, y, z, d);
	}
	return coarse_at<CG>(Lc, AD, x, y, z, d);
}
template <bool CG, bool SPH, typename T>
__device__ __forceinline__ T fill_z(const Lvl &Lc, const Lvl &Lf, const Geo *gf, const T *AD, int x, int y, int z, int d)
{
	if(z & 1)
	{
		if(SPH)
		{
			const int ex = x > 0 ? x - 1 : 0;
			const double x1 = gf[cg_col(Lf, ex, z >= 2 ? z - 2 : 0)].size[2], x2 = gf[cg_col(Lf, ex, z)].size[2];
			return (T)(x2 / (x1 + x2)) * fill_x<CG, SPH>(Lc, Lf, gf, AD, x, y, z - 1, d) +
			       (T)(x1 / (x1 + x2)) * fill_x<CG, SPH>(Lc, Lf, gf, AD, x, y, z + 1, d);
		}
		return (T)0.5 * fill_x<CG, SPH>(Lc, Lf, gf, AD, x, y, z - 1, d) + (T)0.5 * fill_x<CG, SPH>(Lc, Lf, gf, AD, x, y, z + 1, d);
	}
	return fill_x<CG, SPH>(Lc, Lf, gf, AD, x, y, z, d);
}
// the y fill's two neighbours share their first element's (x, z) column: 1/2
template <bool CG, bool SPH, typename T>
__device__ __forceinline__ void interp_node(const Lvl &Lc, const Lvl &Lf, const Geo *gf, const T *AD, T *AU, int n)
{
	const int z = n % Lf.noz, x = (n / Lf.noz) % Lf.nox, y = n / (Lf.noz * Lf.nox);
	const unsigned f = cg_vflag(Lf, x, y, z);
#pragma unroll
	for(int d = 0; d < 3; ++d)
	{
		T v;
		if(y & 1)
			v = (T)0.5 * fill_z<CG, SPH>(Lc, Lf, gf, AD, x, y - 1, z, d) + (T)0.5 * fill_z<CG, SPH>(Lc, Lf, gf, AD, x, y + 1, z, d);
		else
			v = fill_z<CG, SPH>(Lc, Lf, gf, AD, x, y, z, d);
		AU[3 * n + d] = ((f >> d) & 1u) ? (T)0 : v;
	}
}
