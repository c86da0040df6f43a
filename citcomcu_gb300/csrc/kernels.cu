// sm_103a kernels for CitcomCU's Stokes / SUPG hot path.
//
// Design (one GPU, whole mesh resident in HBM):
//  * The velocity operator is the node-assembled 27-point block stencil of
//    the reference (n_assemble_del2_u, Element_calculations.c:552-621, whose
//    coefficients construct_node_ks, Construct_arrays.c:359-535, builds) but
//    stored in full (243 coefficients per node) and colour-major
//    structure-of-arrays, so every kernel streams coalesced coefficients and
//    gathers its 27 neighbours node-centred: no atomics anywhere.
//  * The lexicographic node-block Gauss-Seidel (gauss_seidel,
//    General_matrix_functions.c:1160-1361) becomes an 8-colour sweep with the
//    same per-node update (the node's 3 dofs relaxed together with 1/diag).
//  * Restriction / prolongation are node-centred gathers.
//  * Reductions are deterministic: fixed grids, per-block partials, the last
//    block sums partials in block order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "kernels.h"

namespace {

constexpr int TPB = 256;

#include "device.cuh"

inline int nblocks(long n, int tpb = TPB) { return (int)((n + tpb - 1) / tpb); }

template <typename T> __device__ __forceinline__ T ldcs(const T *p) { return __ldcs(p); }



// ---------------------------------------------------------------- reduce

template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], Red red, double *out)
{
	__shared__ double sh[RED_THREADS / 32][NV];
	__shared__ bool last;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
	for(int i = 0; i < NV; ++i)
		for(int o = 16; o > 0; o >>= 1)
			v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
	if(lane == 0)
#pragma unroll
		for(int i = 0; i < NV; ++i)
			sh[warp][i] = v[i];
	__syncthreads();
	if(threadIdx.x == 0)
	{
		for(int i = 0; i < NV; ++i)
		{
			double s = 0.0;
			for(int w = 0; w < (int)(blockDim.x >> 5); ++w)
				s += sh[w][i];
			red.partials[blockIdx.x * NV + i] = s;
		}
		__threadfence();
		const unsigned t = atomicAdd(red.counter, 1u);
		last = (t == gridDim.x - 1);
	}
	__syncthreads();
	if(last)
	{
		__threadfence();
		// fixed-order sum of the partials by the last block
		for(int i = 0; i < NV; ++i)
		{
			double s = 0.0;
			for(int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
				s += __ldcg(red.partials + b * NV + i);
			for(int o = 16; o > 0; o >>= 1)
				s += __shfl_down_sync(0xffffffffu, s, o);
			if(lane == 0)
				sh[warp][0] = s;
			__syncthreads();
			if(threadIdx.x == 0)
			{
				double t = 0.0;
				for(int w = 0; w < (int)(blockDim.x >> 5); ++w)
					t += sh[w][0];
				out[i] = t;
			}
			__syncthreads();
		}
		if(threadIdx.x == 0)
			*red.counter = 0u;
	}
}

inline int red_grid(long n)
{
	int g = nblocks(n, RED_THREADS);
	return g < 1 ? 1 : (g > RED_MAX_BLOCKS ? RED_MAX_BLOCKS : g);
}

// ---------------------------------------------------------------- assemble

// One thread per node (colour-major position): builds the node's 27 3x3
// blocks from the elements it shares with each neighbour.  K_e follows
// get_elt_k's Cartesian branch (Element_calculations.c:223-247) plus the
// augmented-Lagrangian term of get_aug_k (:1127-1163); rows of constrained
// dofs and columns of constrained neighbour dofs are zero
// (construct_node_ks, Construct_arrays.c:409-505); BI = 1/diag of the
// unmasked K (build_diagonal_of_K, Element_calculations.c:624-652).
__global__ void k_assemble(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ evi, int aug, double lambda,
                           double *__restrict__ K64, float *__restrict__ K32, double *__restrict__ BI64, float *__restrict__ BI32)
{
	pdl_begin();
	const int p = blockIdx.x * blockDim.x + threadIdx.x;
	if(p >= L.nno)
		return;
	const int c = colour_of_pos(L, p);
	int x, y, z;
	cg_decode(L, c, p - L.coff[c], x, y, z);
	const unsigned fn = cg_vflag(L, x, y, z);
	double diag[3] = {0.0, 0.0, 0.0};

	for(int s = 0; s < 27; ++s)
	{
		const int dz = s % 3 - 1, dx = (s / 3) % 3 - 1, dy = s / 9 - 1;
		double blk[9];
#pragma unroll
		for(int q = 0; q < 9; ++q)
			blk[q] = 0.0;
		const int mx = x + dx, my = y + dy, mz = z + dz;
		const bool inside = mx >= 0 && mx < L.nox && my >= 0 && my < L.noy && mz >= 0 && mz < L.noz;
		if(inside)
		{
			const unsigned fm = cg_vflag(L, mx, my, mz);
			// elements holding both n and m: corner (ox,oy,oz) of n with (o+d) in {0,1}
			for(int oy = 0; oy < 2; ++oy)
			{
				if(oy + dy < 0 || oy + dy > 1 || y - oy < 0 || y - oy >= L.ely)
					continue;
				for(int ox = 0; ox < 2; ++ox)
				{
					if(ox + dx < 0 || ox + dx > 1 || x - ox < 0 || x - ox >= L.elx)
						continue;
					for(int oz = 0; oz < 2; ++oz)
					{
						if(oz + dz < 0 || oz + dz > 1 || z - oz < 0 || z - oz >= L.elz)
							continue;
						const int e = (z - oz) + L.elz * ((x - ox) + L.elx * (y - oy));
						const Geo *G = geo + cg_col(L, x - ox, z - oz);
						const int a = cg_local_index(ox, oy, oz);
						const int b = cg_local_index(ox + dx, oy + dy, oz + dz);
						double eta[8], mean = 0.0;
#pragma unroll
						for(int k = 0; k < 8; ++k)
						{
							eta[k] = evi[8 * e + k];
							mean += eta[k];
						}
						mean *= 0.125;
#pragma unroll
						for(int q = 0; q < 9; ++q)
						{
							double v = 0.0;
#pragma unroll
							for(int k = 0; k < 8; ++k)
								v += eta[k] * G->Mk[k][a][b][q];
							if(aug)
								v += mean * lambda * G->g[3 * a + q / 3] * G->g[3 * b + q % 3];
							blk[q] += v;
						}
						if(s == 13)
						{
							// unmasked diagonal for BI
#pragma unroll
							for(int i = 0; i < 3; ++i)
							{
								double v = 0.0;
#pragma unroll
								for(int k = 0; k < 8; ++k)
									v += eta[k] * G->Mk[k][a][a][4 * i];
								if(aug)
									v += mean * lambda * G->g[3 * a + i] * G->g[3 * a + i];
								diag[i] += v;
							}
						}
					}
				}
			}
#pragma unroll
			for(int i = 0; i < 3; ++i)
#pragma unroll
				for(int j = 0; j < 3; ++j)
					if(((fn >> i) & 1u) || ((fm >> j) & 1u))
						blk[3 * i + j] = 0.0;
		}
#pragma unroll
		for(int i = 0; i < 3; ++i)
#pragma unroll
			for(int j = 0; j < 3; ++j)
			{
				const size_t off = cg_kidx(L, s, i, j, p);
				if(K64)
					K64[off] = blk[3 * i + j];
				if(K32)
					K32[off] = (float)blk[3 * i + j];
			}
	}
#pragma unroll
	for(int i = 0; i < 3; ++i)
	{
		const double bi = 1.0 / diag[i];
		if(BI64)
			BI64[3 * (size_t)p + i] = bi;
		if(BI32)
			BI32[3 * (size_t)p + i] = (float)bi;
	}
}

// build_diagonal_of_Ahat / assemble_dAhatp_entry (Element_calculations.c:654-689, 771-829)
__global__ void k_bpi(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ BI, double *__restrict__ BPI, int precond)
{
	pdl_begin();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	if(!precond)
	{
		BPI[e] = 1.0;
		return;
	}
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const Geo *G = geo + cg_col(L, ex, ez);
	double bu = 0.0;
	for(int a = 0; a < 8; ++a)
	{
		const int p = cg_pos(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2));
#pragma unroll
		for(int i = 0; i < 3; ++i)
		{
			const double g = G->g[3 * a + i];
			bu += g * g * BI[3 * (size_t)p + i];
		}
	}
	BPI[e] = (bu != 0.0) ? 1.0 / bu : 1.0;
}

// ---------------------------------------------------------------- stencil

// Stencil products are computed by one thread per (node, neighbour slot): a
// block holds NB = 16 nodes x 27 slots; each warp covers two slots of 16
// consecutive nodes of one colour.  Each thread issues its 9 coefficient loads
// and 3 neighbour loads at once (memory-level parallelism instead of a long
// per-node gather), writes the 3 partial row sums to shared memory, and 96
// threads then add the 27 partials of each (node, row).  Neighbours outside
// the mesh are clamped onto it; their coefficients are zero.
constexpr int NB = 16;
constexpr int SLOT_THREADS = 27 * NB;  // 432

// coordinates of the node at colour-major position p
// partial row sums of slot s of the node at (x,y,z), position p
template <typename T, bool STREAM>
__device__ __forceinline__ void slot_partial(const Lvl &L, const T *K, const T *u, int p, int x, int y, int z, int s, T &a0,
                                             T &a1, T &a2)
{
	const int dz = s % 3 - 1, dx = (s / 3) % 3 - 1, dy = s / 9 - 1;
	const int m = cg_node(L, clampi(x + dx, 0, L.nox - 1), clampi(y + dy, 0, L.noy - 1), clampi(z + dz, 0, L.noz - 1));
	T k[9];  // k[3j + i] = K_{n,m}[i][j]
	if(L.aos)
	{
		const T *kc = K + (size_t)243 * p + s;
#pragma unroll
		for(int i = 0; i < 3; ++i)
#pragma unroll
			for(int j = 0; j < 3; ++j)
				k[3 * j + i] = kc[27 * (3 * i + j)];
	}
	else
	{
		const size_t s3 = 3 * (size_t)L.npad;
		const T *kc = K + (size_t)(3 * s) * s3 + 3 * (size_t)p;  // group (3s + j), row i at +i
#pragma unroll
		for(int j = 0; j < 3; ++j)
#pragma unroll
			for(int i = 0; i < 3; ++i)
				k[3 * j + i] = STREAM ? ldcs(kc + j * s3 + i) : kc[j * s3 + i];
	}
	const T u0 = u[3 * m], u1 = u[3 * m + 1], u2 = u[3 * m + 2];
	a0 = k[0] * u0 + k[3] * u1 + k[6] * u2;
	a1 = k[1] * u0 + k[4] * u1 + k[7] * u2;
	a2 = k[2] * u0 + k[5] * u1 + k[8] * u2;
}

// Shared-memory layout of the partial sums: part[(s * 3 + i) * NB + ln]
template <typename T> struct SlotSmem
{
	T part[27 * 3 * NB];
};

// Computes r_i = sum_m K_{n,m}[i][:] u_m for the NB nodes at colour-major
// positions p0 .. p0+cnt-1 (all of one colour); on return the threads
// t < 3*cnt hold (node t/3, row t%3) in `row`.  Every thread of the block
// must call it (it synchronises).
template <typename T, bool STREAM>
__device__ __forceinline__ void block_rows(const Lvl &L, const T *K, const T *u, int p0, int cnt, T *part, T &row)
{
	const int ln = threadIdx.x % NB, s = threadIdx.x / NB;
	if(ln < cnt)
	{
		int c, x, y, z;
		pos_xyz(L, p0 + ln, c, x, y, z);
		T a0, a1, a2;
		slot_partial<T, STREAM>(L, K, u, p0 + ln, x, y, z, s, a0, a1, a2);
		part[(s * 3 + 0) * NB + ln] = a0;
		part[(s * 3 + 1) * NB + ln] = a1;
		part[(s * 3 + 2) * NB + ln] = a2;
	}
	__syncthreads();
	row = 0;
	if((int)threadIdx.x < 3 * cnt)
	{
		const int q = threadIdx.x / 3, i = threadIdx.x % 3;
		T acc = 0;
#pragma unroll
		for(int ss = 0; ss < 27; ++ss)
			acc += part[(ss * 3 + i) * NB + q];
		row = acc;
	}
}

// node index of the (node, row) owner thread t < 3*cnt of a slot block
__device__ __forceinline__ int row_owner_node(const Lvl &L, int p0)
{
	int c, x, y, z;
	pos_xyz(L, p0 + (int)threadIdx.x / 3, c, x, y, z);
	return cg_node(L, x, y, z);
}

// MODE 0: out = K u;  MODE 1: out = f - K u.  One block per NB nodes of a colour; grid (blocks, colours).
// The owner threads fetch their f before the gather so that its latency overlaps.
template <typename T, int MODE>
__global__ void __launch_bounds__(SLOT_THREADS) k_kmul(Lvl L, const T *__restrict__ K, const T *__restrict__ u, const T *__restrict__ f,
                                                       T *__restrict__ out)
{
	pdl_begin();
	__shared__ SlotSmem<T> sm;
	const int c = blockIdx.y;
	const int nc = L.coff[c + 1] - L.coff[c];
	const int q0 = blockIdx.x * NB;
	if(q0 >= nc)
		return;
	const int cnt = min(NB, nc - q0);
	const int p0 = L.coff[c] + q0;
	const bool owner = (int)threadIdx.x < 3 * cnt;
	const int i = threadIdx.x % 3;
	int n = 0;
	T fi = 0;
	if(owner)
	{
		n = row_owner_node(L, p0);
		if(MODE == 1)
			fi = f[3 * n + i];
	}
	T r;
	block_rows<T, true>(L, K, u, p0, cnt, sm.part, r);
	if(owner)
		out[3 * n + i] = (MODE == 1) ? fi - r : r;
}

// a.b and a.a in FP64 (a = AU, b = res for the line search of multi_grid,
// General_matrix_functions.c:626-630): out2[0] = a.b, out2[1] = a.a
// FP32 vectors: each thread sums its products in FP32 over runs of 8 of its
// elements and adds each run's sums in FP64.  Converting and accumulating
// every element in FP64 would make GB300's FP64 pipe, not HBM, the bound
// (four FP64 operations per element: about 20 us on the finest level).
template <typename T>
__global__ void k_dot2(int n, const T *__restrict__ a, const T *__restrict__ b, Red red, double *out2)
{
	pdl_begin();
	double v[2] = {0.0, 0.0};
	const int stride = gridDim.x * blockDim.x;
	if constexpr(sizeof(T) == 4)
	{
		int i = blockIdx.x * blockDim.x + threadIdx.x;
		while(i < n)
		{
			float s0 = 0.f, s1 = 0.f;
#pragma unroll
			for(int k = 0; k < 8; ++k, i += stride)
				if(i < n)
				{
					const float x = a[i];
					s0 = fmaf(x, b[i], s0);
					s1 = fmaf(x, x, s1);
				}
			v[0] += (double)s0;
			v[1] += (double)s1;
		}
	}
	else
		for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
		{
			const double x = a[i];
			v[0] += x * (double)b[i];
			v[1] += x * x;
		}
	block_reduce_store<2>(v, red, out2);
}

// vel += alpha del ; res -= alpha AU (finest level only); alpha = num/den,
// formed once per block (an FP64 division per element would cost more than
// the kernel's memory traffic on GB300) and applied in the vectors' precision
template <typename T>
__global__ void k_vel_update(int n, T *__restrict__ vel, const T *__restrict__ del, T *__restrict__ res, const T *__restrict__ AU,
                             const double *__restrict__ nd, int update_res)
{
	pdl_begin();
	__shared__ double s_alpha;
	if(threadIdx.x == 0)
		s_alpha = nd[0] / nd[1];
	__syncthreads();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n)
		return;
	const T alpha = (T)s_alpha;
	vel[i] += alpha * del[i];
	if(update_res)
		res[i] -= alpha * AU[i];
}

// One Gauss-Seidel colour: d_n += (F_n - sum_m K_{n,m} d_m) o BI_n.  The three
// rows of a node are relaxed together from the same d (the reference's
// "Jacobi at a node"): all reads happen before the block's barrier.  The
// owner of (node, row) fetches F, 1/diag and its own d before the gather, so
// the update needs no second memory round trip.
template <typename T>
__global__ void __launch_bounds__(SLOT_THREADS) k_gs_colour(Lvl L, const T *__restrict__ K, const T *__restrict__ BI,
                                                            const T *__restrict__ F, T *d, int c)
{
	pdl_begin();
	__shared__ SlotSmem<T> sm;
	const int nc = L.coff[c + 1] - L.coff[c];
	const int q0 = blockIdx.x * NB;
	if(q0 >= nc)
		return;
	const int cnt = min(NB, nc - q0);
	const int p0 = L.coff[c] + q0;
	const bool owner = (int)threadIdx.x < 3 * cnt;
	const int i = threadIdx.x % 3;
	int n = 0;
	T fi = 0, bi = 0, di = 0;
	if(owner)
	{
		n = row_owner_node(L, p0);
		fi = F[3 * n + i];
		bi = BI[3 * (size_t)(p0 + (int)threadIdx.x / 3) + i];
		di = d[3 * n + i];
	}
	T r;
	block_rows<T, true>(L, K, d, p0, cnt, sm.part, r);
	if(owner)
		d[3 * n + i] = di + (fi - r) * bi;
}

// All sweeps and colours of one gauss_seidel call on a small level (stored
// node by node) in one CTA of 32 warps: a warp relaxes one node at a time,
// lane s < 27 handling neighbour slot s (9 coefficients and 3 neighbour
// values), the 27 partial rows added by warp shuffles; lanes 0..2 then apply
// the node update.  The node and neighbour indices of every (position, slot)
// are computed once into a shared-memory table, so a colour phase is loads,
// 9 FMAs and the shuffles.  STAGE 2: stencil, 1/diag, F and d staged in
// shared memory as well (coarsest levels); STAGE 1: 1/diag, F and d staged,
// the stencil read through L2 (it does not depend on the colour phase, so a
// phase costs one L2 round trip); each warp processes up to GSW nodes at once.
constexpr int GS_WARPS = 32;
constexpr int GSW = 3;
template <typename T, int STAGE>
__global__ void __launch_bounds__(GS_WARPS * 32) k_gs_small(Lvl L, const T *__restrict__ K, const T *__restrict__ BI,
                                                            const T *__restrict__ F, T *d, int cycles, int zero_start)
{
	pdl_begin();
	extern __shared__ __align__(16) unsigned char smem_raw[];
	// neighbour table: nb[28 * p + s] = neighbour node of slot s (clamped), nb[28 * p + 27] = node of position p
	int *nb = reinterpret_cast<int *>(smem_raw);
	T *tail = reinterpret_cast<T *>(smem_raw + (((size_t)28 * L.nno * sizeof(int) + 15) / 16) * 16);
	for(int t = threadIdx.x; t < 28 * L.nno; t += blockDim.x)
	{
		const int p = t / 28, s = t - 28 * p;
		int c, x, y, z;
		pos_xyz(L, p, c, x, y, z);
		if(s == 27)
			nb[t] = cg_node(L, x, y, z);
		else
		{
			const int dz = s % 3 - 1, dx = (s / 3) % 3 - 1, dy = s / 9 - 1;
			nb[t] = cg_node(L, clampi(x + dx, 0, L.nox - 1), clampi(y + dy, 0, L.noy - 1), clampi(z + dz, 0, L.noz - 1));
		}
	}
	const T *Kp = K, *Bp = BI, *Fp = F;
	T *dp = d;
	if(STAGE > 0)
	{
		T *sK = tail;                                         // 243 * nno when STAGE == 2
		T *sB = sK + (STAGE == 2 ? (size_t)243 * L.nno : 0);  // 3 * nno
		T *sF = sB + (size_t)3 * L.nno;                       // neq
		T *sd = sF + L.neq;                                   // neq
		if(STAGE == 2)
		{
			// 16-byte words, eight loads in flight per thread before the stores
			// (K comes from cudaMalloc and sK is 16-byte aligned)
			const int nk = 243 * L.nno;
			const int n16 = (int)(((size_t)nk * sizeof(T)) / 16);
			const uint4 *src = reinterpret_cast<const uint4 *>(K);
			uint4 *dst = reinterpret_cast<uint4 *>(sK);
			for(int b = threadIdx.x; b < n16; b += 8 * blockDim.x)
			{
				uint4 v[8];
#pragma unroll
				for(int k = 0; k < 8; ++k)
					if(b + k * (int)blockDim.x < n16)
						v[k] = __ldg(src + b + k * blockDim.x);
#pragma unroll
				for(int k = 0; k < 8; ++k)
					if(b + k * (int)blockDim.x < n16)
						dst[b + k * blockDim.x] = v[k];
			}
			for(int i = n16 * (int)(16 / sizeof(T)) + threadIdx.x; i < nk; i += blockDim.x)
				sK[i] = K[i];
			Kp = sK;
		}
		for(int i = threadIdx.x; i < 3 * L.nno; i += blockDim.x)
			sB[i] = BI[i];
		for(int i = threadIdx.x; i < L.neq; i += blockDim.x)
		{
			sF[i] = F[i];
			sd[i] = zero_start ? (T)0 : d[i];
		}
		Bp = sB;
		Fp = sF;
		dp = sd;
	}
	else if(zero_start)
		for(int i = threadIdx.x; i < L.neq; i += blockDim.x)
			d[i] = 0;
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int s = lane < 27 ? lane : 13;  // idle lanes shadow the centre slot with zero weight
	const T wgt = lane < 27 ? (T)1 : (T)0;
	for(int cyc = 0; cyc < cycles; ++cyc)
		for(int c = 0; c < 8; ++c)
		{
			const int nc = L.coff[c + 1] - L.coff[c];
			for(int q0 = warp; q0 < nc; q0 += GS_WARPS * GSW)
			{
				T r[GSW][3];
				int nn[GSW], pp[GSW];
#pragma unroll
				for(int w = 0; w < GSW; ++w)
				{
					const int q = q0 + w * GS_WARPS;
					r[w][0] = r[w][1] = r[w][2] = 0;
					nn[w] = -1;
					pp[w] = 0;
					if(q < nc)
					{
						const int p = L.coff[c] + q;
						const int m = nb[28 * p + s];
						const T *kc = Kp + (size_t)243 * p + s;
						const T u0 = dp[3 * m], u1 = dp[3 * m + 1], u2 = dp[3 * m + 2];
						r[w][0] = wgt * (kc[0] * u0 + kc[27] * u1 + kc[54] * u2);
						r[w][1] = wgt * (kc[81] * u0 + kc[108] * u1 + kc[135] * u2);
						r[w][2] = wgt * (kc[162] * u0 + kc[189] * u1 + kc[216] * u2);
						nn[w] = nb[28 * p + 27];
						pp[w] = p;
					}
				}
#pragma unroll
				for(int w = 0; w < GSW; ++w)
				{
					if(q0 + w * GS_WARPS >= nc)
						break;  // warp-uniform
#pragma unroll
					for(int i = 0; i < 3; ++i)
						for(int o = 16; o > 0; o >>= 1)
							r[w][i] += __shfl_xor_sync(0xffffffffu, r[w][i], o);
				}
#pragma unroll
				for(int w = 0; w < GSW; ++w)
					if(nn[w] >= 0 && lane < 3)
					{
						const T ri = lane == 0 ? r[w][0] : (lane == 1 ? r[w][1] : r[w][2]);
						dp[3 * nn[w] + lane] += (Fp[3 * nn[w] + lane] - ri) * Bp[3 * (size_t)pp[w] + lane];
					}
			}
			__syncthreads();
		}
	if(STAGE > 0)
		for(int i = threadIdx.x; i < L.neq; i += blockDim.x)
			d[i] = dp[i];
}

// All sweeps of one gauss_seidel call on a small FP32 level (up to about a
// thousand nodes) in one CTA: three nodes per warp (27 lanes), all warps on
// the nodes of one colour, a barrier between colours.  KS: the padded
// stencil is staged in shared memory (coarsest levels), else read through L2
// in every phase.  All threads stage; only the first `nwork` warps relax,
// synchronising on a named barrier, and the others leave.
template <bool KS>
__global__ void __launch_bounds__(1024) k_gs_tiny(Lvl L, const float4 *__restrict__ Kt, const float *__restrict__ BI,
                                                  const float *__restrict__ F, float *d, int cycles, int zero_start, int nwork)
{
	pdl_begin();
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int HZ = L.noz + 2, HXZ = (L.nox + 2) * HZ, HN = HXZ * (L.noy + 2);
	float4 *sK = reinterpret_cast<float4 *>(smem_raw);     // 63 * nno when KS
	float4 *sd = sK + (KS ? (size_t)63 * L.nno : 0);         // halo grid, (d_x, d_y, d_z, 0)
	float4 *sF = sd + HN;                                    // (F_x, F_y, F_z, 0) of position p
	float4 *sB = sF + L.nno;                                 // 1/diag of position p
	int *shp = reinterpret_cast<int *>(sB + L.nno);          // halo index of position p
	if(KS)
	{
		const int n16 = 63 * L.nno;
		for(int b = threadIdx.x; b < n16; b += 4 * blockDim.x)
		{
			float4 v[4];
#pragma unroll
			for(int k = 0; k < 4; ++k)
				if(b + k * (int)blockDim.x < n16)
					v[k] = __ldg(Kt + b + k * blockDim.x);
#pragma unroll
			for(int k = 0; k < 4; ++k)
				if(b + k * (int)blockDim.x < n16)
					sK[b + k * blockDim.x] = v[k];
		}
	}
	for(int t = threadIdx.x; t < HN; t += blockDim.x)
		sd[t] = make_float4(0.f, 0.f, 0.f, 0.f);
	for(int p = threadIdx.x; p < L.nno; p += blockDim.x)
		sB[p] = make_float4(BI[3 * p], BI[3 * p + 1], BI[3 * p + 2], 0.f);
	__syncthreads();
	for(int n = threadIdx.x; n < L.nno; n += blockDim.x)
	{
		const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
		const int p = cg_pos(L, x, y, z), hp = (z + 1) + HZ * (x + 1) + HXZ * (y + 1);
		shp[p] = hp;
		sF[p] = make_float4(F[3 * n], F[3 * n + 1], F[3 * n + 2], 0.f);
		if(!zero_start)
			sd[hp] = make_float4(d[3 * n], d[3 * n + 1], d[3 * n + 2], 0.f);
	}
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	if(warp >= nwork)
		return;
	const int nthr = 32 * nwork;
	const int sub = lane / 9, r9 = lane - 9 * sub;
	// first of the lane's three neighbour cells relative to the node
	const int uoff = -1 + HZ * (r9 % 3 - 1) + HXZ * (r9 / 3 - 1);
	const float4 *Kb = KS ? sK : Kt;
	for(int cyc = 0; cyc < cycles; ++cyc)
		for(int c = 0; c < 8; ++c)
		{
			const int c0 = L.coff[c], nc = L.coff[c + 1] - c0;
			for(int q0 = 3 * warp; q0 < nc; q0 += 3 * nwork)
			{
				const int q = q0 + sub;
				const bool active = lane < 27 && q < nc;
				const int p = c0 + (active ? q : 0);
				float r0 = 0.f, r1 = 0.f, r2 = 0.f;
				int hp = 0;
				if(active)
				{
					hp = shp[p];
					const float4 *kr = Kb + (size_t)63 * p + 7 * r9;
					if(KS)
						kt_rows(kr, sd + hp + uoff, r0, r1, r2);
					else
					{
						float4 kg[7];
#pragma unroll
						for(int t = 0; t < 7; ++t)
							kg[t] = __ldg(kr + t);
						kt_rows(kg, sd + hp + uoff, r0, r1, r2);
					}
				}
				r0 = kt_sum9(r0, lane);
				r1 = kt_sum9(r1, lane);
				r2 = kt_sum9(r2, lane);
				if(active && r9 == 0)
				{
					float4 dv = sd[hp];
					const float4 f = sF[p], bi = sB[p];
					dv.x += (f.x - r0) * bi.x;
					dv.y += (f.y - r1) * bi.y;
					dv.z += (f.z - r2) * bi.z;
					sd[hp] = dv;
				}
			}
			asm volatile("bar.sync 1, %0;" ::"r"(nthr) : "memory");
		}
	for(int n = threadIdx.x; n < L.nno; n += nthr)
	{
		const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
		const float4 v = sd[(z + 1) + HZ * (x + 1) + HXZ * (y + 1)];
		d[3 * n] = v.x;
		d[3 * n + 1] = v.y;
		d[3 * n + 2] = v.z;
	}
}

// the padded stencil from the node-by-node FP32 stencil (one thread per word)
__global__ void k_tiny_stencil(Lvl L, const float *__restrict__ K, float *__restrict__ Kt)
{
	pdl_begin();
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if(t >= KT_WORDS * L.nno)
		return;
	const int p = t / KT_WORDS, w = t - KT_WORDS * p, r9 = w / 28, e = w - 28 * r9;
	float v = 0.f;
	if(e < 27)
	{
		const int k = e / 9, i = (e / 3) % 3, j = e % 3;
		v = K[cg_kidx(L, 3 * r9 + k, i, j, p)];
	}
	Kt[t] = v;
}

// ---------------------------------------------------------------- transfers

template <typename T>
__global__ void k_project(Lvl Lf, Lvl Lc, const Geo *__restrict__ gc, const T *__restrict__ AU, T *__restrict__ AD)
{
	pdl_begin();
	// sums in the level's own precision: FP64 for the FP64 path; FP32 for the
	// FP32 multigrid (as in the cluster program), where FP64 arithmetic would
	// run at GB300's low FP64 rate
	project_lanes<false, T, T>(Lf, Lc, gc, AU, AD, blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T, bool SPH>
__global__ void k_interp(Lvl Lc, Lvl Lf, const Geo *__restrict__ gf, const T *__restrict__ AD, T *__restrict__ AU)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n < Lf.nno)
		interp_node<false, SPH, T>(Lc, Lf, gf, AD, AU, n);
}

// ---------------------------------------------------------------- div / grad

// assemble_div_u (Element_calculations.c:691-722)
__global__ void k_div(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ U, double *__restrict__ divU)
{
	pdl_begin();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const Geo *G = geo + cg_col(L, ex, ez);
	double s = 0.0;
#pragma unroll
	for(int a = 0; a < 8; ++a)
	{
		const int n = cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2));
		s += G->g[3 * a] * U[3 * n] + G->g[3 * a + 1] * U[3 * n + 1] + G->g[3 * a + 2] * U[3 * n + 2];
	}
	divU[e] = s;
}

// assemble_grad_p (Element_calculations.c:727-769) as a node-centred gather
__global__ void k_grad(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ P, double *__restrict__ gradP)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
	double g0 = 0.0, g1 = 0.0, g2 = 0.0;
	for(int a = 0; a < 8; ++a)
	{
		const int ex = x - cg_loc(a, 0), ey = y - cg_loc(a, 1), ez = z - cg_loc(a, 2);
		if(ex < 0 || ex >= L.elx || ey < 0 || ey >= L.ely || ez < 0 || ez >= L.elz)
			continue;
		const double p = P[ez + L.elz * (ex + L.elx * ey)];
		const Geo *G = geo + cg_col(L, ex, ez);
		g0 += G->g[3 * a] * p;
		g1 += G->g[3 * a + 1] * p;
		g2 += G->g[3 * a + 2] * p;
	}
	const unsigned f = cg_vflag(L, x, y, z);
	gradP[3 * n] = (f & 1u) ? 0.0 : g0;
	gradP[3 * n + 1] = (f & 2u) ? 0.0 : g1;
	gradP[3 * n + 2] = (f & 4u) ? 0.0 : g2;
}

__global__ void k_strip(Lvl L, double *r)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
	const unsigned f = cg_vflag(L, x, y, z);
	for(int d = 0; d < 3; ++d)
		if((f >> d) & 1u)
			r[3 * n + d] = 0.0;
}

// ---------------------------------------------------------------- vectors

__global__ void k_dot(int n, const double *__restrict__ a, const double *__restrict__ b, Red red, double *out)
{
	pdl_begin();
	double v[1] = {0.0};
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		v[0] += a[i] * b[i];
	block_reduce_store<1>(v, red, out);
}

__global__ void k_dots4(int n, const double *a0, const double *b0, const double *a1, const double *b1, const double *a2,
                        const double *b2, const double *a3, const double *b3, Red red, double *out)
{
	pdl_begin();
	double v[4] = {0.0, 0.0, 0.0, 0.0};
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		if(a0)
			v[0] += a0[i] * b0[i];
		if(a1)
			v[1] += a1[i] * b1[i];
		if(a2)
			v[2] += a2[i] * b2[i];
		if(a3)
			v[3] += a3[i] * b3[i];
	}
	block_reduce_store<4>(v, red, out);
}

__global__ void k_axpby(int n, double *y, double a, const double *x, double b)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
		y[i] = a * y[i] + b * x[i];
}

__global__ void k_mul(int n, double *z, const double *a, const double *b)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
		z[i] = a[i] * b[i];
}

// ------------------------------------------------ Uzawa iteration (device scalars)
// The scalars of one iteration of solve_Ahat_p_fhat (Stokes_flow_Incomp.c:393-446)
// stay on the device: sc[0] = r1.z1, sc[1] = previous r1.z1 (= r0.z0),
// sc[2] = s2.Ahat, sc[3] = alpha, sc[4] = error flag.

// z1 = BPI o r1 and r1.z1 -> sc[0]
__global__ void k_uz_precond(int n, const double *__restrict__ BPI, const double *__restrict__ r1, double *__restrict__ z1,
                             Red red, double *sc)
{
	pdl_begin();
	double v[1] = {0.0};
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const double z = BPI[i] * r1[i];
		z1[i] = z;
		v[0] += r1[i] * z;
	}
	block_reduce_store<1>(v, red, sc);
}

// s2 = z1 (first iteration) or z1 + (r1.z1 / r0.z0) s1; a zero r0.z0 sets the error flag
__global__ void k_uz_search(int n, double *__restrict__ s2, const double *__restrict__ z1, const double *__restrict__ s1,
                            double *sc, int first)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	double delta = 0.0;
	if(!first)
	{
		if(sc[1] == 0.0)
		{
			if(i == 0)
				sc[4] = 1.0;
		}
		else
			delta = sc[0] / sc[1];
	}
	if(i < n)
		s2[i] = first ? z1[i] : z1[i] + delta * s1[i];
}

// alpha = valid ? r1.z1 / s2.Ahat : 0;  r2 = r1 - alpha Ahat;  P += alpha s2
__global__ void k_uz_update_p(int n, double *__restrict__ r2, const double *__restrict__ r1, const double *__restrict__ Ah,
                              double *__restrict__ P, const double *__restrict__ s2, double *sc, int valid)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const double alpha = valid ? sc[0] / sc[2] : 0.0;
	if(i < n)
	{
		r2[i] = r1[i] - alpha * Ah[i];
		P[i] += alpha * s2[i];
	}
}

// V -= alpha u1; the last kernel of the iteration also records alpha and
// moves r1.z1 into the r0.z0 slot for the next iteration
__global__ void k_uz_update_v(int n, double *__restrict__ V, const double *__restrict__ u1, double *sc, int valid)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const double alpha = valid ? sc[0] / sc[2] : 0.0;
	if(i < n)
		V[i] -= alpha * u1[i];
}

__global__ void k_uz_finish(double *sc, int valid)
{
	pdl_begin();
	if(threadIdx.x == 0 && blockIdx.x == 0)
	{
		sc[3] = valid ? sc[0] / sc[2] : 0.0;
		sc[1] = sc[0];
	}
}

__global__ void k_lin2(int n, double *z, double a, const double *x, double b, const double *y)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
		z[i] = a * x[i] + b * y[i];
}

__global__ void k_sub3(int n, double *z, const double *f, const double *a, const double *b)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
		z[i] = f[i] - a[i] - b[i];
}

__global__ void k_d2f(int n, float *dst, const double *src)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
		dst[i] = (float)src[i];
}

__global__ void k_add_f2d(int n, double *dst, const float *src)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
		dst[i] += (double)src[i];
}

// ---------------------------------------------------------------- viscosity

// visc_from_T, rheol 3 (Viscosity_structures.c:617-646) or visc_from_mat
// (:477-489), with VMAX/VMIN (:414-427) and the material group of the element
// centroid (construct_mat_group, Construct_arrays.c:742-800)
__global__ void k_visc_from_T(Lvl L, const Geo *__restrict__ geo, Rheo r, const double *__restrict__ T, double *__restrict__ evi)
{
	pdl_begin();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const double zc = L.org[2] + ((double)ez + 0.5) * L.h[2];
	const Geo *G = geo + cg_col(L, ex, ez);
	int layer = 0;
	for(int i = 0; i < r.num_mat - 1; ++i)
		if(zc >= r.z_layer[i])
		{
			layer = i + 1;
			break;
		}
	if(!layer)
		layer = r.num_mat;
	const int m = layer - 1;
	double TT[8];
#pragma unroll
	for(int a = 0; a < 8; ++a)
	{
		const double t = T[cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2))];
		TT[a] = t > 0.0 ? t : 0.0;
	}
#pragma unroll
	for(int k = 0; k < 8; ++k)
	{
		double v;
		if(r.tdepv)
		{
			double t = 1.0e-32;
#pragma unroll
			for(int a = 0; a < 8; ++a)
				t += TT[a] * G->N[k][a];
			v = r.visc0[m] * exp(r.viscE[m] * (r.viscT[m] - t));
		}
		else
			v = r.visc0[m];
		if(!r.sdepv)
		{
			if(r.vmax_on && v > r.vmax)
				v = r.vmax;
			if(r.vmin_on && v < r.vmin)
				v = r.vmin;
		}
		evi[8 * e + k] = v;
	}
}

// strain_rate_2_inv (Viscosity_structures.c:979-1086) at the element centre,
// SQRT form: sqrt(0.5 sum of e_ij e_ij).  The spherical branch forms its
// tensor from the velocity gradient in (theta, phi, r) as the reference does
// (diagonal 2 d_ii, off-diagonal d_ij + d_ji).
__global__ void k_strain_rate(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ V, double *__restrict__ edot)
{
	pdl_begin();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const Geo *G = geo + cg_col(L, ex, ez);
	double vv[8][3];
	for(int a = 0; a < 8; ++a)
	{
		const int n = cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2));
		for(int d = 0; d < 3; ++d)
			vv[a][d] = V[(size_t)d * L.nno + n];
	}
	double e11, e22, e33, e12, e13, e23;
	if(!L.sphere)
	{
		double du[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
		for(int a = 0; a < 8; ++a)
			for(int p = 0; p < 3; ++p)
				for(int q = 0; q < 3; ++q)
					du[p][q] += vv[a][p] * G->gnxc[a][q];
		e11 = du[0][0];
		e22 = du[1][1];
		e33 = du[2][2];
		e12 = 0.5 * (du[0][1] + du[1][0]);
		e13 = 0.5 * (du[0][2] + du[2][0]);
		e23 = 0.5 * (du[1][2] + du[2][1]);
	}
	else
	{
		const double ra = G->rinvc, st = sin(G->thetac), ct = cos(G->thetac), n = 0.125;
		double x1 = 0, x2 = 0, x3 = 0, x4 = 0, x5 = 0, x6 = 0;
		for(int a = 0; a < 8; ++a)
		{
			const double v1 = vv[a][0], v2 = vv[a][1], v3 = vv[a][2];
			const double g0 = G->gnxc[a][0], g1 = G->gnxc[a][1], g2 = G->gnxc[a][2];
			x1 += (v1 * g0 + v3 * n) * ra;
			x2 += ((v2 * g1 + v1 * n * ct) / st + v3 * n) * ra;
			x3 += v3 * g2;
			x4 += ((v1 * g1 - v2 * n * ct) / st + v2 * g0) * ra;
			x5 += v1 * g2 + ra * (v3 * g0 - v1 * n);
			x6 += v2 * g2 + ra * (v3 * g1 / st - v2 * n);
		}
		e11 = 2.0 * x1;
		e22 = 2.0 * x2;
		e33 = 2.0 * x3;
		e12 = x4;
		e13 = x5;
		e23 = x6;
	}
	const double s = e11 * e11 + e12 * e12 * 2.0 + e22 * e22 + e23 * e23 * 2.0 + e33 * e33 + e13 * e13 * 2.0;
	edot[e] = sqrt(0.5 * s);
}

// visc_from_S (Viscosity_structures.c:744-846), rheology 1 (eta <- 2 eta /
// (1 + s eta^(1-1/n))) or 2 (eta <- eta / (1 + s eta^(1-1/n)) below the
// transition temperature; without composition), s = (2 edot / trns)^(1-1/n)
// of the element's material; then VMAX/VMIN (:414-427).  edot null: 1.
__global__ void k_visc_from_S(Lvl L, const Geo *__restrict__ geo, Rheo r, const double *__restrict__ T,
                              const double *__restrict__ edot, double *__restrict__ evi)
{
	pdl_begin();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const Geo *G = geo + cg_col(L, ex, ez);
	const double zc = L.org[2] + ((double)ez + 0.5) * L.h[2];
	int layer = 0;
	for(int i = 0; i < r.num_mat - 1; ++i)
		if(zc >= r.z_layer[i])
		{
			layer = i + 1;
			break;
		}
	if(!layer)
		layer = r.num_mat;
	const int m = layer - 1;
	const double ed = edot ? edot[e] : 1.0;
	const double e1 = 1.0 - 1.0 / r.sdepv_expt[m];
	const double scale = pow(2.0 * ed / r.sdepv_trns[m], e1);
	double TT[8];
	for(int a = 0; a < 8; ++a)
	{
		const double t = T[cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2))];
		TT[a] = t > 0.0 ? t : 0.0;
	}
	for(int k = 0; k < 8; ++k)
	{
		double v = evi[8 * e + k];
		if(r.sdepv_rheology == 1)
			v = 2.0 * v / (1.0 + scale * pow(v, e1));
		else
		{
			double t = 0.0;
			for(int a = 0; a < 8; ++a)
				t += TT[a] * G->N[k][a];
			// the transition temperature (3000) and composition (2) of the
			// reference's defaults: the non-dimensional T and C = 0 are below
			if(t < 3000.0)
				v = v / (1.0 + scale * pow(v, e1));
		}
		if(r.vmax_on && v > r.vmax)
			v = r.vmax;
		if(r.vmin_on && v < r.vmin)
			v = r.vmin;
		evi[8 * e + k] = v;
	}
}

// visc_from_gint_to_nodes (Nodal_mesh.c:583-615)
__global__ void k_visc_to_nodes(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ evi, double *__restrict__ VN)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
	double s = 0.0, m = 0.0;
	for(int a = 0; a < 8; ++a)
	{
		const int ex = x - cg_loc(a, 0), ey = y - cg_loc(a, 1), ez = z - cg_loc(a, 2);
		if(ex < 0 || ex >= L.elx || ey < 0 || ey >= L.ely || ez < 0 || ez >= L.elz)
			continue;
		const int e = ez + L.elz * (ex + L.elx * ey);
		const double w = geo[cg_col(L, ex, ez)].tww[a];
		double t = 0.0;
		for(int k = 0; k < 8; ++k)
			t += evi[8 * e + k];
		s += w * (t / 8.0);
		m += w;
	}
	VN[n] = s * (1.0 / m);
}

// project_scalar (Solver_multigrid.c:338-394)
__global__ void k_project_scalar(Lvl Lf, Lvl Lc, const Geo *__restrict__ geoc, const double *__restrict__ VN, double *__restrict__ VD)
{
	pdl_begin();
	const int N = blockIdx.x * blockDim.x + threadIdx.x;
	if(N >= Lc.nno)
		return;
	const int Z = N % Lc.noz, X = (N / Lc.noz) % Lc.nox, Y = N / (Lc.noz * Lc.nox);
	double s = 0.0, m = 0.0;
	for(int a = 0; a < 8; ++a)
	{
		const int ox = cg_loc(a, 0), oy = cg_loc(a, 1), oz = cg_loc(a, 2);
		const int ex = X - ox, ey = Y - oy, ez = Z - oz;
		if(ex < 0 || ex >= Lc.elx || ey < 0 || ey >= Lc.ely || ez < 0 || ez >= Lc.elz)
			continue;
		const double w = geoc[cg_col(Lc, ex, ez)].tww[a];
		m += w;
		double t = 0.0;
		for(int b = 0; b < 8; ++b)
			t += VN[cg_node(Lf, 2 * ex + ox + cg_loc(b, 0), 2 * ey + oy + cg_loc(b, 1), 2 * ez + oz + cg_loc(b, 2))];
		s += (t / 8.0) * w;
	}
	VD[N] = s * (1.0 / m);
}

// visc_from_nodes_to_gint (Nodal_mesh.c:617-640)
__global__ void k_visc_to_gint(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ VN, double *__restrict__ evi)
{
	pdl_begin();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const Geo *G = geo + cg_col(L, ex, ez);
	double v[8];
#pragma unroll
	for(int a = 0; a < 8; ++a)
		v[a] = VN[cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2))];
#pragma unroll
	for(int k = 0; k < 8; ++k)
	{
		double t = 0.0;
#pragma unroll
		for(int a = 0; a < 8; ++a)
			t += G->N[k][a] * v[a];
		evi[8 * e + k] = t;
	}
}

// ---------------------------------------------------------------- forces

// return_horiz_ave (Global_operations.c:133-251) of Ra*T, one block per z
// layer: the lower faces of the layer's elements (the top node layer takes the
// top elements' lower-face weights, as the reference does)
__global__ void k_horiz_ave(Lvl L, const Geo *__restrict__ geo, double Ra, const double *__restrict__ T, double *__restrict__ H)
{
	pdl_begin();
	const int z = blockIdx.x;
	__shared__ double sh[2][TPB / 32];
	double s = 0.0, w = 0.0;
	const double dg = L.h[0] * L.h[1] / 4.0;
	const int ez = z < L.elz ? z : L.elz - 1;
	for(int i = threadIdx.x; i < L.elx * L.ely; i += blockDim.x)
	{
		const int x = i % L.elx, y = i / L.elx;
		if(L.sphere)
		{
			const double *wf = geo[cg_col(L, x, ez)].wface;
			s += Ra * T[cg_node(L, x, y, z)] * wf[0] + Ra * T[cg_node(L, x + 1, y, z)] * wf[1] +
			     Ra * T[cg_node(L, x + 1, y + 1, z)] * wf[2] + Ra * T[cg_node(L, x, y + 1, z)] * wf[3];
			w += wf[0] + wf[1] + wf[2] + wf[3];
			continue;
		}
		s += dg * (Ra * T[cg_node(L, x, y, z)] + Ra * T[cg_node(L, x + 1, y, z)] + Ra * T[cg_node(L, x + 1, y + 1, z)] +
		           Ra * T[cg_node(L, x, y + 1, z)]);
		w += 4.0 * dg;
	}
	for(int o = 16; o > 0; o >>= 1)
	{
		s += __shfl_down_sync(0xffffffffu, s, o);
		w += __shfl_down_sync(0xffffffffu, w, o);
	}
	if((threadIdx.x & 31) == 0)
	{
		sh[0][threadIdx.x >> 5] = s;
		sh[1][threadIdx.x >> 5] = w;
	}
	__syncthreads();
	if(threadIdx.x == 0)
	{
		double a = 0.0, b = 0.0;
		for(int k = 0; k < (int)(blockDim.x >> 5); ++k)
		{
			a += sh[0][k];
			b += sh[1][k];
		}
		H[z] = a / b;
	}
}

// thermal_buoyancy (Pan_problem_misc_functions.c:83-156): Ra*T minus the layer mean
__global__ void k_buoyancy(Lvl L, double Ra, const double *__restrict__ T, const double *__restrict__ H, double *__restrict__ b)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n < L.nno)
		b[n] = Ra * T[n] - H[n % L.noz];
}

// assemble_forces + get_elt_f (Element_calculations.c:74-125, 989-1120), node-centred, stripped
__global__ void k_forces(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ buoy, double *__restrict__ F)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
	double fn[3] = {0.0, 0.0, 0.0};
	for(int a = 0; a < 8; ++a)
	{
		const int ex = x - cg_loc(a, 0), ey = y - cg_loc(a, 1), ez = z - cg_loc(a, 2);
		if(ex < 0 || ex >= L.elx || ey < 0 || ey >= L.ely || ez < 0 || ez >= L.elz)
			continue;
		const Geo *G = geo + cg_col(L, ex, ez);
		double bb[8];
		for(int b = 0; b < 8; ++b)
			bb[b] = buoy[cg_node(L, ex + cg_loc(b, 0), ey + cg_loc(b, 1), ez + cg_loc(b, 2))];
		double s[3] = {0.0, 0.0, 0.0};
		for(int k = 0; k < 8; ++k)
		{
			double fg = 0.0;
			for(int b = 0; b < 8; ++b)
				fg += bb[b] * G->N[k][b];
			// the radial force of the Gauss point on node a's components
			// (Cartesian: z only; spherical: Cc(3, i, a, k), :1086)
			const double w = fg * G->N[k][a] * G->gda[k];
			for(int i = 0; i < 3; ++i)
				s[i] += w * G->cr[k][a][i];
		}
		for(int i = 0; i < 3; ++i)
			fn[i] += s[i];
	}
	const unsigned f = cg_vflag(L, x, y, z);
	F[3 * n] = (f & 1u) ? 0.0 : fn[0];
	F[3 * n + 1] = (f & 2u) ? 0.0 : fn[1];
	F[3 * n + 2] = (f & 4u) ? 0.0 : fn[2];
}

// The same forces for the box.  There the force is vertical and an element
// contributes J sum_k N_ka N_kb b_b to node a: its consistent mass matrix,
// which for 2x2x2 Gauss points is the tensor product of the 1D matrix
// [[c0, c1], [c1, c0]], c0 = P^2 + Q^2 = 2/3, c1 = 2 P Q = 1/3 (P, Q the 1D
// shape function values at the Gauss points).  Summed over the elements
// around a node it stays a product of 1D weights: (c1, 2 c0, c1) inside,
// (c0, c1) at a wall.  27 FMA per node instead of about a thousand.
__global__ void k_forces_box(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ buoy, double *__restrict__ F)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
	constexpr double P = 0.5 * (1.0 + 0.57735026918962576451), Q = 0.5 * (1.0 - 0.57735026918962576451);
	const double c0 = P * P + Q * Q, c1 = 2.0 * P * Q;
	auto w1 = [&](int i, int ni, int d) {
		// 1D weight of neighbour offset d (-1, 0, 1) at index i of ni
		if(d < 0)
			return i > 0 ? c1 : 0.0;
		if(d > 0)
			return i < ni - 1 ? c1 : 0.0;
		return (i > 0 ? c0 : 0.0) + (i < ni - 1 ? c0 : 0.0);
	};
	double s = 0.0;
	for(int dy = -1; dy <= 1; ++dy)
	{
		const double wy = w1(y, L.noy, dy);
		if(wy == 0.0)
			continue;
		for(int dx = -1; dx <= 1; ++dx)
		{
			const double wxy = wy * w1(x, L.nox, dx);
			if(wxy == 0.0)
				continue;
			const int col = cg_node(L, x + dx, y + dy, 0);
			for(int dz = -1; dz <= 1; ++dz)
			{
				const double wz = w1(z, L.noz, dz);
				if(wz != 0.0)
					s += wxy * wz * buoy[col + z + dz];
			}
		}
	}
	const unsigned f = cg_vflag(L, x, y, z);
	F[3 * n] = 0.0;
	F[3 * n + 1] = 0.0;
	F[3 * n + 2] = (f & 4u) ? 0.0 : geo->gda[0] * s;
}

// v_from_vector (Stokes_flow_Incomp.c:530-553): V[d*nno + n]; constrained dofs take VB = 0
__global__ void k_v_from_vector(Lvl L, const double *__restrict__ U, double *__restrict__ V)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
	const unsigned f = cg_vflag(L, x, y, z);
	for(int d = 0; d < 3; ++d)
		V[(size_t)d * L.nno + n] = ((f >> d) & 1u) ? 0.0 : U[3 * n + d];
}

// ---------------------------------------------------------------- energy

__device__ __forceinline__ bool t_dirichlet(const Lvl &L, int n) { int z = n % L.noz; return z == 0 || z == L.noz - 1; }

// pg_solver's per-element work: pg_shape_fn (Advection_diffusion.c:448-555)
// and element_residual (:564-727), diffusivity 1, Q = Q0; the spherical
// branches scale the theta and phi derivatives by 1/r and 1/(r sin theta)
// (:506-529, 620-641, 668-674), 1 in the box
__global__ void k_pg_residual(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ T, const double *__restrict__ Tdot,
                              const double *__restrict__ V, double Q0, double *__restrict__ Eres)
{
	pdl_begin();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const Geo *G = geo + cg_col(L, ex, ez);
	const double diff = 1.0, twodiff = 2.0 * diff;
	double vn[8][3], tn[8], dtn[8];
#pragma unroll
	for(int a = 0; a < 8; ++a)
	{
		const int n = cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2));
		vn[a][0] = V[n];
		vn[a][1] = V[(size_t)L.nno + n];
		vn[a][2] = V[2 * (size_t)L.nno + n];
		tn[a] = T[n];
		dtn[a] = t_dirichlet(L, n) ? 0.0 : Tdot[n];
	}
	double uc[3] = {0.0, 0.0, 0.0};
#pragma unroll
	for(int a = 0; a < 8; ++a)
#pragma unroll
		for(int d = 0; d < 3; ++d)
			uc[d] += 0.125 * vn[a][d];
	double us[3], up[3];
#pragma unroll
	for(int d = 0; d < 3; ++d)
	{
		us[d] = fabs(uc[d] * G->size[d]);
		up[d] = (us[d] > twodiff) ? (1.0 - twodiff / us[d]) : 0.0;
	}
	const double unorm = uc[0] * uc[0] + uc[1] * uc[1] + uc[2] * uc[2];
	const double adiff = (unorm > 0.000001) ? ((us[0] * up[0] + us[1] * up[1] + us[2] * up[2]) / (2.0 * unorm)) : 0.0;
	double er[8];
#pragma unroll
	for(int a = 0; a < 8; ++a)
		er[a] = 0.0;
#pragma unroll
	for(int k = 0; k < 8; ++k)
	{
		double v0 = 0, v1 = 0, v2 = 0, t0 = 0, t1 = 0, t2 = 0, dT = 0;
		const double ri = G->rinv[k], rs = G->rsin[k], jk = G->gda[k];
#pragma unroll
		for(int a = 0; a < 8; ++a)
		{
			const double Nk = G->N[k][a];
			dT += dtn[a] * Nk;
			v0 += vn[a][0] * Nk;
			v1 += vn[a][1] * Nk;
			v2 += vn[a][2] * Nk;
			t0 += G->gnx[k][a][0] * tn[a] * ri;
			t1 += G->gnx[k][a][1] * tn[a] * rs;
			t2 += G->gnx[k][a][2] * tn[a];
		}
		const double adv = dT - Q0 + v0 * t0 + v1 * t1 + v2 * t2;
#pragma unroll
		for(int a = 0; a < 8; ++a)
		{
			const double g0 = G->gnx[k][a][0], g1 = G->gnx[k][a][1], g2 = G->gnx[k][a][2];
			const double pg = G->N[k][a] + adiff * (v0 * g0 * ri + v1 * g1 * rs + v2 * g2);
			er[a] -= pg * jk * adv + diff * jk * (g0 * t0 * ri + g1 * t1 * rs + g2 * t2);
		}
	}
#pragma unroll
	for(int a = 0; a < 8; ++a)
		Eres[8 * (size_t)e + a] = er[a];
}

// The same residual for the box, sum-factorised.  A box element's shape
// functions are products of 1D factors, (1 + s xi)/2 along each axis: P =
// (1 + beta)/2 where the Gauss point (xi = +-beta) and the node (s = +-1) lie
// on the same side, Q = (1 - beta)/2 otherwise, and dN/dx_d has +-1/h_d in
// place of the factor along d.  So
//  * values at the 2x2x2 Gauss points are three passes of 1D interpolation
//    (ip3), and the test sum over the Gauss points against N_a is the same
//    operator (the 1D factor matrix is symmetric);
//  * the derivative along d is the difference of the two d-faces, bilinearly
//    interpolated to the other two axes' Gauss points: the same at both Gauss
//    points along d;
//  * the test against dN_a/dx_d sums the Gauss points along d first.
// With jk = |J| w constant, er[a] = -jk (sum_k N_ka A_k + sum_d sum_k
// dN_a/dx_d(k) B_kd), A_k = dT - Q0 + v.grad T (the advection residual),
// B_kd = adiff A_k v_d + diff dT/dx_d (the upwind and diffusion fluxes).
// About 550 FP64 operations per element instead of about 1,750: the kernel
// is bound by GB300's FP64 rate.  Index q = x + 2 y + 4 z of the element's
// nodes and Gauss points.
namespace pgbox {
constexpr double P = 0.5 * (1.0 + 0.57735026918962576451), Q = 0.5 * (1.0 - 0.57735026918962576451);

// f at the Gauss points (in place): 1D passes along x, y, z
__device__ __forceinline__ void ip3(double f[8])
{
#pragma unroll
	for(int s = 1; s <= 4; s <<= 1)
#pragma unroll
		for(int q = 0; q < 8; ++q)
			if(!(q & s))
			{
				const double a = f[q], b = f[q + s];
				f[q] = P * a + Q * b;
				f[q + s] = Q * a + P * b;
			}
}

// 2x2 bilinear pass (in place), stride s1 then s2 within a 4-array
__device__ __forceinline__ void ip2(double g[4])
{
#pragma unroll
	for(int s = 1; s <= 2; s <<= 1)
#pragma unroll
		for(int q = 0; q < 4; ++q)
			if(!(q & s))
			{
				const double a = g[q], b = g[q + s];
				g[q] = P * a + Q * b;
				g[q + s] = Q * a + P * b;
			}
}

// the two axes other than d, in increasing order, and their strides in q
__device__ __forceinline__ int q_of(int d, int lo, int hi, int side)
{
	// node/Gauss point with coordinate `side` along d, lo along the lower
	// other axis, hi along the higher one
	const int a1 = d == 0 ? 1 : 0, a2 = d == 2 ? 1 : 2;
	return (side << d) | (lo << a1) | (hi << a2);
}
} // namespace pgbox

__global__ void __launch_bounds__(128) k_pg_residual_box(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ T,
                                                         const double *__restrict__ Tdot, const double *__restrict__ V,
                                                         double Q0, double *__restrict__ Eres)
{
	pdl_begin();
	using namespace pgbox;
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const Geo *G = geo;
	const double diff = 1.0, twodiff = 2.0 * diff;
	const double jk = G->gda[0];
	const double ih[3] = {1.0 / L.h[0], 1.0 / L.h[1], 1.0 / L.h[2]};
	const int n0 = cg_node(L, ex, ey, ez);
	const int sx = L.noz, sy = L.noz * L.nox;  // node strides along x and y (z: 1)
	auto node = [&](int q) { return n0 + (q & 1) * sx + ((q >> 1) & 1) * sy + ((q >> 2) & 1); };
	// grad T at the Gauss points: gt[d][lo + 2 hi] (the same at both Gauss points along d)
	double gt[3][4];
	{
		double tn[8];
#pragma unroll
		for(int q = 0; q < 8; ++q)
			tn[q] = T[node(q)];
#pragma unroll
		for(int d = 0; d < 3; ++d)
		{
#pragma unroll
			for(int m = 0; m < 4; ++m)
				gt[d][m] = (tn[q_of(d, m & 1, m >> 1, 1)] - tn[q_of(d, m & 1, m >> 1, 0)]) * ih[d];
			ip2(gt[d]);
		}
	}
	// dT/dt at the Gauss points (fixed-temperature nodes contribute 0)
	double dt[8];
#pragma unroll
	for(int q = 0; q < 8; ++q)
	{
		const int n = node(q);
		dt[q] = t_dirichlet(L, n) ? 0.0 : Tdot[n];
	}
	ip3(dt);
	// velocity at the nodes, its element mean (the upwind parameter), then at the Gauss points
	double vk[3][8];
#pragma unroll
	for(int q = 0; q < 8; ++q)
	{
		const int n = node(q);
		vk[0][q] = V[n];
		vk[1][q] = V[(size_t)L.nno + n];
		vk[2][q] = V[2 * (size_t)L.nno + n];
	}
	double uc[3];
#pragma unroll
	for(int d = 0; d < 3; ++d)
	{
		double s = 0.0;
#pragma unroll
		for(int q = 0; q < 8; ++q)
			s += vk[d][q];
		uc[d] = 0.125 * s;
	}
	double us[3], up[3];
#pragma unroll
	for(int d = 0; d < 3; ++d)
	{
		us[d] = fabs(uc[d] * G->size[d]);
		up[d] = (us[d] > twodiff) ? (1.0 - twodiff / us[d]) : 0.0;
	}
	const double unorm = uc[0] * uc[0] + uc[1] * uc[1] + uc[2] * uc[2];
	const double adiff = (unorm > 0.000001) ? ((us[0] * up[0] + us[1] * up[1] + us[2] * up[2]) / (2.0 * unorm)) : 0.0;
#pragma unroll
	for(int d = 0; d < 3; ++d)
		ip3(vk[d]);
	// A_k in dt (in place); the fluxes B_kd summed over the Gauss points along d: sb[d][lo + 2 hi]
	double sb[3][4];
#pragma unroll
	for(int d = 0; d < 3; ++d)
#pragma unroll
		for(int m = 0; m < 4; ++m)
			sb[d][m] = 0.0;
#pragma unroll
	for(int q = 0; q < 8; ++q)
	{
		const int x = q & 1, y = (q >> 1) & 1, z = q >> 2;
		const double gx = gt[0][y + 2 * z], gy = gt[1][x + 2 * z], gz = gt[2][x + 2 * y];
		const double A = dt[q] - Q0 + vk[0][q] * gx + vk[1][q] * gy + vk[2][q] * gz;
		dt[q] = A;
		const double aa = adiff * A;
		sb[0][y + 2 * z] += aa * vk[0][q] + diff * gx;
		sb[1][x + 2 * z] += aa * vk[1][q] + diff * gy;
		sb[2][x + 2 * y] += aa * vk[2][q] + diff * gz;
	}
	ip3(dt);  // sum_k N_ka A_k at the nodes
#pragma unroll
	for(int d = 0; d < 3; ++d)
		ip2(sb[d]);
	double er[8];
#pragma unroll
	for(int q = 0; q < 8; ++q)
	{
		const int x = q & 1, y = (q >> 1) & 1, z = q >> 2;
		const double fx = x ? sb[0][y + 2 * z] : -sb[0][y + 2 * z];
		const double fy = y ? sb[1][x + 2 * z] : -sb[1][x + 2 * z];
		const double fz = z ? sb[2][x + 2 * y] : -sb[2][x + 2 * y];
		er[q] = -jk * (dt[q] + fx * ih[0] + fy * ih[1] + fz * ih[2]);
	}
	// element-local node order a (cg_loc) of the residual vector
#pragma unroll
	for(int a = 0; a < 8; ++a)
		Eres[8 * (size_t)e + a] = er[cg_loc(a, 0) + 2 * cg_loc(a, 1) + 4 * cg_loc(a, 2)];
}

// DTdot = (sum of element residuals at the node) / lumped mass
__global__ void k_pg_gather(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ Eres, double *__restrict__ DTdot)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
	double s = 0.0, m = 0.0;
	for(int a = 0; a < 8; ++a)
	{
		const int ex = x - cg_loc(a, 0), ey = y - cg_loc(a, 1), ez = z - cg_loc(a, 2);
		if(ex < 0 || ex >= L.elx || ey < 0 || ey >= L.ely || ez < 0 || ez >= L.elz)
			continue;
		s += Eres[8 * (size_t)(ez + L.elz * (ex + L.elx * ey)) + a];
		m += geo[cg_col(L, ex, ez)].tww[a];
	}
	DTdot[n] = s * (1.0 / m);
}

// predictor (Advection_diffusion.c:352-367)
__global__ void k_predictor(Lvl L, double *T, double *Tdot, double dt, double gamma)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	if(!t_dirichlet(L, n))
		T[n] += (1.0 - gamma) * dt * Tdot[n];
	Tdot[n] = 0.0;
}

// corrector (Advection_diffusion.c:369-386)
__global__ void k_corrector(Lvl L, double *T, double *Tdot, const double *DTdot, double dt, double gamma)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	if(!t_dirichlet(L, n))
		T[n] += gamma * dt * DTdot[n];
	Tdot[n] += DTdot[n];
}

// temperatures_conform_bcs (Boundary_conditions.c:949-991): T = 1 at the bottom, 0 at the top
__global__ void k_conform_T(Lvl L, double *T)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz;
	if(z == 0)
		T[n] = 1.0;
	else if(z == L.noz - 1)
		T[n] = 0.0;
}

// max (Tmax, Global_operations.c:394-407) reported through the sum machinery as -min(-x)
__global__ void k_max(int n, const double *__restrict__ T, Red red, double *out)
{
	pdl_begin();
	__shared__ double sh[RED_THREADS / 32];
	__shared__ bool last;
	double m = -10.0;
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		m = fmax(m, T[i]);
	for(int o = 16; o > 0; o >>= 1)
		m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
	if((threadIdx.x & 31) == 0)
		sh[threadIdx.x >> 5] = m;
	__syncthreads();
	if(threadIdx.x == 0)
	{
		double t = -10.0;
		for(int w = 0; w < (int)(blockDim.x >> 5); ++w)
			t = fmax(t, sh[w]);
		red.partials[blockIdx.x] = t;
		__threadfence();
		last = (atomicAdd(red.counter, 1u) == gridDim.x - 1);
	}
	__syncthreads();
	if(last && threadIdx.x == 0)
	{
		__threadfence();
		double t = -10.0;
		for(int b = 0; b < (int)gridDim.x; ++b)
			t = fmax(t, __ldcg(red.partials + b));
		out[0] = t;
		*red.counter = 0u;
	}
}

// advective part of std_timestep (Advection_diffusion.c:737-810): min over elements of 0.5/uc
__global__ void k_adv_step(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ V, Red red, double *out)
{
	pdl_begin();
	__shared__ double sh[RED_THREADS / 32];
	__shared__ bool last;
	double m = 1.0e8;
	for(int e = blockIdx.x * blockDim.x + threadIdx.x; e < L.nel; e += gridDim.x * blockDim.x)
	{
		const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
		double uc[3] = {0.0, 0.0, 0.0};
		for(int a = 0; a < 8; ++a)
		{
			const int n = cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2));
			for(int d = 0; d < 3; ++d)
				uc[d] += 0.125 * V[(size_t)d * L.nno + n];
		}
		const Geo *G = geo + cg_col(L, ex, ez);
		const double u = fabs(uc[0]) / G->size[0] + fabs(uc[1]) / G->size[1] + fabs(uc[2]) / G->size[2];
		m = fmin(m, 0.5 / u);
	}
	for(int o = 16; o > 0; o >>= 1)
		m = fmin(m, __shfl_down_sync(0xffffffffu, m, o));
	if((threadIdx.x & 31) == 0)
		sh[threadIdx.x >> 5] = m;
	__syncthreads();
	if(threadIdx.x == 0)
	{
		double t = 1.0e8;
		for(int w = 0; w < (int)(blockDim.x >> 5); ++w)
			t = fmin(t, sh[w]);
		red.partials[blockIdx.x] = t;
		__threadfence();
		last = (atomicAdd(red.counter, 1u) == gridDim.x - 1);
	}
	__syncthreads();
	if(last && threadIdx.x == 0)
	{
		__threadfence();
		double t = 1.0e8;
		for(int b = 0; b < (int)gridDim.x; ++b)
			t = fmin(t, __ldcg(red.partials + b));
		out[0] = t;
		*red.counter = 0u;
	}
}

// ---------------------------------------------------------------- observables

// heat_flux (Process_buoyancy.c:63-203), step 1: element mean of u_z T - dT/dz
__global__ void k_hf_elem(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ T, const double *__restrict__ V,
                          double *__restrict__ uTe)
{
	pdl_begin();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const Geo *G = geo + cg_col(L, ex, ez);
	double vz[8], tt[8];
	for(int a = 0; a < 8; ++a)
	{
		const int n = cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2));
		vz[a] = V[2 * (size_t)L.nno + n];
		tt[a] = T[n];
	}
	double uT = 0.0;
	for(int k = 0; k < 8; ++k)
	{
		double u = 0, t = 0, dz = 0;
		for(int a = 0; a < 8; ++a)
		{
			u += vz[a] * G->N[k][a];
			t += tt[a] * G->N[k][a];
			dz += tt[a] * G->gnx[k][a][2];
		}
		uT += (u * t - dz) * G->gda[k];
	}
	uTe[e] = uT / G->area;
}

// step 2: nodal flux = TWW-weighted element means / lumped mass
__global__ void k_hf_node(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ uTe, double *__restrict__ hf)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
	double s = 0.0, m = 0.0;
	for(int a = 0; a < 8; ++a)
	{
		const int ex = x - cg_loc(a, 0), ey = y - cg_loc(a, 1), ez = z - cg_loc(a, 2);
		if(ex < 0 || ex >= L.elx || ey < 0 || ey >= L.ely || ez < 0 || ez >= L.elz)
			continue;
		const double w = geo[cg_col(L, ex, ez)].tww[a];
		s += w * uTe[ez + L.elz * (ex + L.elx * ey)];
		m += w;
	}
	hf[n] = s * (1.0 / m);
}

// step 3: surface extrapolation 2 hf[s] - hf[s-1], summed over the four nodes of
// each surface element and weighted by the volume of the element below (top)
// or above (bottom) it; out = (top sum, bottom sum, top weight, bottom weight)
__global__ void k_hf_surface(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ hf, Red red, double *out)
{
	pdl_begin();
	double v[4] = {0.0, 0.0, 0.0, 0.0};
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < L.elx * L.ely; i += gridDim.x * blockDim.x)
	{
		const int x = i % L.elx, y = i / L.elx;
		const int xs[4] = {x, x + 1, x + 1, x}, ys[4] = {y, y, y + 1, y + 1};
		double tt = 0.0, tb = 0.0;
		for(int j = 0; j < 4; ++j)
		{
			const int top = cg_node(L, xs[j], ys[j], L.noz - 1), bot = cg_node(L, xs[j], ys[j], 0);
			tt += 2.0 * hf[top] - hf[top - 1];
			tb += 2.0 * hf[bot] - hf[bot + 1];
		}
		const double at = geo[cg_col(L, x, L.elz - 1)].area, ab = geo[cg_col(L, x, 0)].area;
		v[0] += tt * at;
		v[1] += tb * ab;
		v[2] += at;
		v[3] += ab;
	}
	block_reduce_store<4>(v, red, out);
}

// Output fields of heat_flux (Process_buoyancy.c:103-136), per element: the
// Gauss integrals over the element / its area of u_z T - dT/dz, u_z T' and
// u_z |T'|, T' = T - <T> (HT: the layer means of T); ue = 3 x nel
__global__ void k_out_elem(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ T, const double *__restrict__ V,
                           const double *__restrict__ HT, double *__restrict__ ue)
{
	pdl_begin();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= L.nel)
		return;
	const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
	const Geo *G = geo + cg_col(L, ex, ez);
	double vz[8], tt[8], ta[8];
	for(int a = 0; a < 8; ++a)
	{
		const int n = cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2));
		vz[a] = V[2 * (size_t)L.nno + n];
		tt[a] = T[n];
		ta[a] = T[n] - HT[ez + cg_loc(a, 2)];
	}
	double s0 = 0.0, s1 = 0.0, s2 = 0.0;
	for(int k = 0; k < 8; ++k)
	{
		double u = 0, t = 0, t1 = 0, dz = 0;
		for(int a = 0; a < 8; ++a)
		{
			u += vz[a] * G->N[k][a];
			t += tt[a] * G->N[k][a];
			t1 += ta[a] * G->N[k][a];
			dz += tt[a] * G->gnx[k][a][2];
		}
		s0 += (u * t - dz) * G->gda[k];
		s1 += u * t1 * G->gda[k];
		s2 += u * fabs(t1) * G->gda[k];
	}
	ue[e] = s0 / G->area;
	ue[L.nel + e] = s1 / G->area;
	ue[2 * L.nel + e] = s2 / G->area;
}

// nodal fields from the element means, TWW-weighted / lumped mass: f = 3 x nno
// (heatflux, heatflux_adv, flux of Process_buoyancy.c:138-152)
__global__ void k_out_node(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ ue, double *__restrict__ f)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const int z = n % L.noz, x = (n / L.noz) % L.nox, y = n / (L.noz * L.nox);
	double s0 = 0.0, s1 = 0.0, s2 = 0.0, m = 0.0;
	for(int a = 0; a < 8; ++a)
	{
		const int ex = x - cg_loc(a, 0), ey = y - cg_loc(a, 1), ez = z - cg_loc(a, 2);
		if(ex < 0 || ex >= L.elx || ey < 0 || ey >= L.ely || ez < 0 || ez >= L.elz)
			continue;
		const double w = geo[cg_col(L, ex, ez)].tww[a];
		const int e = ez + L.elz * (ex + L.elx * ey);
		s0 += w * ue[e];
		s1 += w * ue[L.nel + e];
		s2 += w * ue[2 * L.nel + e];
		m += w;
	}
	const double im = 1.0 / m;
	f[n] = s0 * im;
	f[L.nno + n] = s1 * im;
	f[2 * (size_t)L.nno + n] = s2 * im;
}

// surface heat flux by linear extrapolation of the two outermost nodes of each
// column (Process_buoyancy.c:154-161): surf = (shflux, bhflux), nsf each, and
// the extrapolated values replace the surface nodes of hf
__global__ void k_out_surface(Lvl L, double *__restrict__ hf, double *__restrict__ surf)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	const int nsf = L.nox * L.noy;
	if(i >= nsf)
		return;
	const int top = i * L.noz + L.noz - 1, bot = i * L.noz;
	const double s = 2.0 * hf[top] - hf[top - 1], b = 2.0 * hf[bot] - hf[bot + 1];
	surf[i] = s;
	surf[nsf + i] = b;
	hf[top] = s;
	hf[bot] = b;
}

// |V|^2 per node (averages, Process_velocity.c:198-209)
__global__ void k_out_speed2(Lvl L, const double *__restrict__ V, double *__restrict__ v2)
{
	pdl_begin();
	const int n = blockIdx.x * blockDim.x + threadIdx.x;
	if(n >= L.nno)
		return;
	const double a = V[n], b = V[L.nno + n], c = V[2 * (size_t)L.nno + n];
	v2[n] = a * a + b * b + c * c;
}

// sums = (Nu top sum, bottom sum, top weight, bottom weight, vrms sum, volume)
// -> scal = (Nut, Nub, Vrms); H[noz .. 2 noz) = sqrt of the layer means of |V|^2
__global__ void k_out_final(Lvl L, const double *__restrict__ sums, double *__restrict__ scal, double *__restrict__ H)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < L.noz)
		H[L.noz + i] = sqrt(H[L.noz + i]);
	if(i == 0)
	{
		scal[0] = sums[0] / (4.0 * sums[2]);
		scal[1] = sums[1] / (4.0 * sums[3]);
		scal[2] = sqrt(sums[4] / sums[5]);
	}
}

__global__ void k_vrms(Lvl L, const Geo *__restrict__ geo, const double *__restrict__ V, Red red, double *out)
{
	pdl_begin();
	double v[2] = {0.0, 0.0};
	for(int e = blockIdx.x * blockDim.x + threadIdx.x; e < L.nel; e += gridDim.x * blockDim.x)
	{
		const int ez = e % L.elz, ex = (e / L.elz) % L.elx, ey = e / (L.elz * L.elx);
		const Geo *G = geo + cg_col(L, ex, ez);
		double vn[8][3];
		for(int a = 0; a < 8; ++a)
		{
			const int n = cg_node(L, ex + cg_loc(a, 0), ey + cg_loc(a, 1), ez + cg_loc(a, 2));
			for(int d = 0; d < 3; ++d)
				vn[a][d] = V[(size_t)d * L.nno + n];
		}
		for(int k = 0; k < 8; ++k)
		{
			double u0 = 0, u1 = 0, u2 = 0;
			for(int a = 0; a < 8; ++a)
			{
				u0 += G->N[k][a] * vn[a][0];
				u1 += G->N[k][a] * vn[a][1];
				u2 += G->N[k][a] * vn[a][2];
			}
			v[0] += G->gda[k] * (u0 * u0 + u1 * u1 + u2 * u2);
			v[1] += G->gda[k];
		}
	}
	block_reduce_store<2>(v, red, out);
}

} // namespace

// ====================================================================== host

unsigned long long g_kernel_launches = 0;
int g_use_pdl = 1;

template <typename... KArgs, typename... Args>
static void launch_k_smem(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args)
{
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = smem;
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = g_use_pdl ? 1 : 0;
	cudaLaunchKernelEx(&cfg, kern, ((KArgs)args)...);
	++g_kernel_launches;
}

template <typename... KArgs, typename... Args>
static void launch_k(void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args)
{
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = 0;
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = g_use_pdl ? 1 : 0;
	cudaLaunchKernelEx(&cfg, kern, ((KArgs)args)...);
	++g_kernel_launches;
}

void geo_fill_host(const Lvl &L, Geo *g)
{
	if(L.sphere)
	{
		geo_fill_sphere(L, g);
		return;
	}
	const double beta = 0.57735026918962576451;
	double gnx[8][8][3], gnxc[8][3];
	for(int k = 0; k <= 8; ++k)
		for(int a = 0; a < 8; ++a)
			for(int d = 0; d < 3; ++d)
			{
				double v = 0.5 * (cg_loc(a, d) ? 1.0 : -1.0) * 2.0 / L.h[d];
				for(int dd = 0; dd < 3; ++dd)
					if(dd != d)
					{
						const double sa = cg_loc(a, dd) ? 1.0 : -1.0;
						const double xi = (k == 8) ? 0.0 : (cg_loc(k, dd) ? beta : -beta);
						v *= 0.5 * (1.0 + sa * xi);
					}
				if(k == 8)
					gnxc[a][d] = v;
				else
					gnx[k][a][d] = v;
			}
	for(int k = 0; k < 8; ++k)
		for(int a = 0; a < 8; ++a)
		{
			double v = 1.0;
			for(int d = 0; d < 3; ++d)
				v *= 0.5 * (1.0 + (cg_loc(a, d) ? 1.0 : -1.0) * (cg_loc(k, d) ? beta : -beta));
			g->N[k][a] = v;
			for(int d = 0; d < 3; ++d)
				g->gnx[k][a][d] = gnx[k][a][d];
		}
	for(int k = 0; k < 8; ++k)
		for(int a = 0; a < 8; ++a)
			for(int b = 0; b < 8; ++b)
			{
				const double s = gnx[k][a][0] * gnx[k][b][0] + gnx[k][a][1] * gnx[k][b][1] + gnx[k][a][2] * gnx[k][b][2];
				for(int i = 0; i < 3; ++i)
					for(int j = 0; j < 3; ++j)
						g->Mk[k][a][b][3 * i + j] = L.J * (gnx[k][a][j] * gnx[k][b][i] + (i == j ? s : 0.0));
			}
	for(int a = 0; a < 8; ++a)
		for(int d = 0; d < 3; ++d)
			g->g[3 * a + d] = -gnxc[a][d] * 8.0 * L.J;
	// box element: |J| is constant, TWW = J, the radial direction is z
	for(int k = 0; k < 8; ++k)
	{
		g->gda[k] = L.J;
		g->rinv[k] = 1.0;
		g->rsin[k] = 1.0;
		for(int a = 0; a < 8; ++a)
			for(int i = 0; i < 3; ++i)
				g->cr[k][a][i] = i == 2 ? 1.0 : 0.0;
	}
	for(int a = 0; a < 8; ++a)
		g->tww[a] = L.J;
	for(int d = 0; d < 3; ++d)
		g->size[d] = L.h[d];
	g->area = 8.0 * L.J;
	for(int i = 0; i < 4; ++i)
		g->wface[i] = L.h[0] * L.h[1] / 4.0;
	for(int a = 0; a < 8; ++a)
		for(int d = 0; d < 3; ++d)
			g->gnxc[a][d] = gnxc[a][d];
	g->rinvc = 1.0;
	g->thetac = 0.0;
}

void launch_assemble(cudaStream_t st, const Lvl &L, const Geo *geo, const double *evi, int aug, double lambda, double *K64,
                     float *K32, double *BI64, float *BI32)
{
	launch_k(k_assemble, nblocks(L.nno, 128), 128, st, L, geo, evi, aug, lambda, K64, K32, BI64, BI32);
}

void launch_bpi(cudaStream_t st, const Lvl &L, const Geo *geo, const double *BI64, double *BPI, int precond)
{
	launch_k(k_bpi, nblocks(L.nel), TPB, st, L, geo, BI64, BPI, precond);
}

static int max_colour(const Lvl &L)
{
	int m = 0;
	for(int c = 0; c < 8; ++c)
		m = (L.coff[c + 1] - L.coff[c]) > m ? (L.coff[c + 1] - L.coff[c]) : m;
	return m;
}

// tiled levels go to the bulk-copy kernels of tile.cu, small levels to the slot kernels here
template <typename T> void launch_kmul(cudaStream_t st, const Lvl &L, const T *K, const T *u, T *Au)
{
	if(!L.aos)
		return launch_tile_kmul<T>(st, L, K, u, Au);
	dim3 grid((max_colour(L) + NB - 1) / NB, 8);
	launch_k(k_kmul<T, 0>, grid, SLOT_THREADS, st, L, K, u, (const T *)nullptr, Au);
}

template <typename T> void launch_residual(cudaStream_t st, const Lvl &L, const T *K, const T *f, const T *u, T *r)
{
	if(!L.aos)
		return launch_tile_residual<T>(st, L, K, f, u, r);
	dim3 grid((max_colour(L) + NB - 1) / NB, 8);
	launch_k(k_kmul<T, 1>, grid, SLOT_THREADS, st, L, K, u, f, r);
}

template <typename T>
void launch_kmul_linesearch(cudaStream_t st, const Lvl &L, const T *K, const T *u, const T *res, T *Au, Red red, double *out2)
{
	launch_kmul<T>(st, L, K, u, Au);
	launch_k(k_dot2<T>, red_grid(L.neq), RED_THREADS, st, L.neq, (const T *)Au, res, red, out2);
}

template <typename T> void launch_gs_colour(cudaStream_t st, const Lvl &L, const T *K, const T *BI, const T *F, T *d, int c)
{
	if(!L.aos)
		return launch_tile_gs<T>(st, L, K, BI, F, d, c);
	const int n = L.coff[c + 1] - L.coff[c];
	if(n > 0)
	{
		launch_k(k_gs_colour<T>, (n + NB - 1) / NB, SLOT_THREADS, st, L, K, BI, F, d, c);
	}
}

// The single-CTA smoother serves the small FP32 levels.  In FP64 the one SM
// it runs on is limited by GB300's FP64 rate, so FP64 small levels use the
// all-SM colour launches instead.
bool gs_small_fits(const Lvl &L, size_t word)
{
	return L.aos != 0 && word == sizeof(float) && (((size_t)28 * L.nno * sizeof(int) + 15) / 16) * 16 <= 200 * 1024;
}

static size_t gs_table_bytes(const Lvl &L) { return (((size_t)28 * L.nno * sizeof(int) + 15) / 16) * 16; }
static size_t gs_smem_bytes(const Lvl &L, size_t word, int stage)
{
	return gs_table_bytes(L) + word * ((stage == 2 ? (size_t)243 * L.nno : 0) + (stage > 0 ? 3 * (size_t)L.nno + 2 * (size_t)L.neq : 0));
}
constexpr size_t GS_SMEM_MAX = 200 * 1024;

// k_gs_tiny: [padded stencil], halo-padded correction vector, F, 1/diag, halo index
static size_t gs_tiny_bytes(const Lvl &L, bool ks)
{
	const size_t hn = (size_t)(L.nox + 2) * (L.noy + 2) * (L.noz + 2);
	return (ks ? (size_t)KT_WORDS * L.nno * sizeof(float) : 0) + hn * 16 + (size_t)2 * L.nno * 16 + (size_t)L.nno * sizeof(int);
}

bool gs_tiny_fits(const Lvl &L, size_t word)
{
	return L.aos != 0 && word == sizeof(float) && gs_tiny_bytes(L, false) <= GS_SMEM_MAX;
}

int kernels_init()
{
	// opt in to large dynamic shared memory once, outside any stream capture
	cudaError_t e[5];
	e[0] = cudaFuncSetAttribute(k_gs_small<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GS_SMEM_MAX);
	e[1] = cudaFuncSetAttribute(k_gs_small<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GS_SMEM_MAX);
	e[2] = cudaFuncSetAttribute(k_gs_small<float, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GS_SMEM_MAX);
	e[3] = cudaFuncSetAttribute(k_gs_tiny<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GS_SMEM_MAX);
	e[4] = cudaFuncSetAttribute(k_gs_tiny<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GS_SMEM_MAX);
	for(cudaError_t x : e)
		if(x != cudaSuccess)
			return -1;
	return tile_init();
}

void launch_tiny_stencil(cudaStream_t st, const Lvl &L, const float *K32, float4 *Kt)
{
	launch_k(k_tiny_stencil, nblocks(KT_WORDS * (long)L.nno), TPB, st, L, K32, reinterpret_cast<float *>(Kt));
}

void launch_gs_tiny(cudaStream_t st, const Lvl &L, const float4 *Kt, const float *BI, const float *F, float *d, int cycles,
                    int zero_start)
{
	int maxc = 0;
	for(int c = 0; c < 8; ++c)
		maxc = std::max(maxc, L.coff[c + 1] - L.coff[c]);
	const int nwork = std::max(1, std::min(32, (maxc + 2) / 3));
	if(gs_tiny_bytes(L, true) <= GS_SMEM_MAX)
		launch_k_smem(k_gs_tiny<true>, dim3(1), dim3(1024), gs_tiny_bytes(L, true), st, L, Kt, BI, F, d, cycles, zero_start, nwork);
	else
		launch_k_smem(k_gs_tiny<false>, dim3(1), dim3(1024), gs_tiny_bytes(L, false), st, L, Kt, BI, F, d, cycles, zero_start,
		              nwork);
}

template <typename T>
void launch_gs_small(cudaStream_t st, const Lvl &L, const T *K, const T *BI, const T *F, T *d, int cycles, int zero_start)
{
	const dim3 g(1), b(GS_WARPS * 32);
	if(gs_smem_bytes(L, sizeof(T), 2) <= GS_SMEM_MAX)
		launch_k_smem(k_gs_small<T, 2>, g, b, gs_smem_bytes(L, sizeof(T), 2), st, L, K, BI, F, d, cycles, zero_start);
	else if(gs_smem_bytes(L, sizeof(T), 1) <= GS_SMEM_MAX)
		launch_k_smem(k_gs_small<T, 1>, g, b, gs_smem_bytes(L, sizeof(T), 1), st, L, K, BI, F, d, cycles, zero_start);
	else
		launch_k_smem(k_gs_small<T, 0>, g, b, gs_table_bytes(L), st, L, K, BI, F, d, cycles, zero_start);
}

template <typename T> void launch_project(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, const Geo *gc, const T *AU, T *AD)
{
	launch_k(k_project<T>, nblocks(8 * (long)Lc.nno), TPB, st, Lf, Lc, gc, AU, AD);
}

template <typename T> void launch_interp(cudaStream_t st, const Lvl &Lc, const Lvl &Lf, const Geo *gf, const T *AD, T *AU)
{
	if(Lf.sphere)
		launch_k(k_interp<T, true>, nblocks(Lf.nno), TPB, st, Lc, Lf, gf, AD, AU);
	else
		launch_k(k_interp<T, false>, nblocks(Lf.nno), TPB, st, Lc, Lf, gf, AD, AU);
}

template <typename T>
void launch_vel_update(cudaStream_t st, int n, T *vel, const T *del, T *res, const T *AU, const double *nd, int update_res)
{
	launch_k(k_vel_update<T>, nblocks(n), TPB, st, n, vel, del, res, AU, nd, update_res);
}

#define INST(T)                                                                                                              \
	template void launch_kmul<T>(cudaStream_t, const Lvl &, const T *, const T *, T *);                                      \
	template void launch_residual<T>(cudaStream_t, const Lvl &, const T *, const T *, const T *, T *);                      \
	template void launch_kmul_linesearch<T>(cudaStream_t, const Lvl &, const T *, const T *, const T *, T *, Red, double *); \
	template void launch_gs_colour<T>(cudaStream_t, const Lvl &, const T *, const T *, const T *, T *, int);                 \
	template void launch_gs_small<T>(cudaStream_t, const Lvl &, const T *, const T *, const T *, T *, int, int);             \
	template void launch_project<T>(cudaStream_t, const Lvl &, const Lvl &, const Geo *, const T *, T *);                    \
	template void launch_interp<T>(cudaStream_t, const Lvl &, const Lvl &, const Geo *, const T *, T *);                     \
	template void launch_vel_update<T>(cudaStream_t, int, T *, const T *, T *, const T *, const double *, int);
INST(double)
INST(float)
#undef INST

void launch_div(cudaStream_t st, const Lvl &L, const Geo *geo, const double *U, double *divU)
{
	launch_k(k_div, nblocks(L.nel), TPB, st, L, geo, U, divU);
}

void launch_grad(cudaStream_t st, const Lvl &L, const Geo *geo, const double *P, double *gradP)
{
	launch_k(k_grad, nblocks(L.nno), TPB, st, L, geo, P, gradP);
}

void launch_strip(cudaStream_t st, const Lvl &L, double *r) { launch_k(k_strip, nblocks(L.nno), TPB, st, L, r); }

void launch_dot(cudaStream_t st, int n, const double *a, const double *b, Red red, double *out)
{
	launch_k(k_dot, red_grid(n), RED_THREADS, st, n, a, b, red, out);
}

void launch_dots4(cudaStream_t st, int n, const double *a0, const double *b0, const double *a1, const double *b1, const double *a2,
                  const double *b2, const double *a3, const double *b3, Red red, double *out)
{
	launch_k(k_dots4, red_grid(n), RED_THREADS, st, n, a0, b0, a1, b1, a2, b2, a3, b3, red, out);
}

void launch_axpby(cudaStream_t st, int n, double *y, double a, const double *x, double b)
{
	launch_k(k_axpby, nblocks(n), TPB, st, n, y, a, x, b);
}

void launch_mul(cudaStream_t st, int n, double *z, const double *a, const double *b) { launch_k(k_mul, nblocks(n), TPB, st, n, z, a, b); }

void launch_uzawa_precond(cudaStream_t st, int n, const double *BPI, const double *r1, double *z1, Red red, double *sc)
{
	launch_k(k_uz_precond, red_grid(n), RED_THREADS, st, n, BPI, r1, z1, red, sc);
}

void launch_uzawa_search(cudaStream_t st, int n, double *s2, const double *z1, const double *s1, double *sc, int first)
{
	launch_k(k_uz_search, nblocks(n), TPB, st, n, s2, z1, s1, sc, first);
}

void launch_uzawa_update(cudaStream_t st, int npno, int neq, double *r2, const double *r1, const double *Ah, double *P,
                         const double *s2, double *V, const double *u1, double *sc, int valid)
{
	launch_k(k_uz_update_p, nblocks(npno), TPB, st, npno, r2, r1, Ah, P, s2, sc, valid);
	launch_k(k_uz_update_v, nblocks(neq), TPB, st, neq, V, u1, sc, valid);
	launch_k(k_uz_finish, 1, 32, st, sc, valid);
}

void launch_lin2(cudaStream_t st, int n, double *z, double a, const double *x, double b, const double *y)
{
	launch_k(k_lin2, nblocks(n), TPB, st, n, z, a, x, b, y);
}

void launch_sub3(cudaStream_t st, int n, double *z, const double *f, const double *a, const double *b)
{
	launch_k(k_sub3, nblocks(n), TPB, st, n, z, f, a, b);
}

void launch_copy_d2f(cudaStream_t st, int n, float *dst, const double *src) { launch_k(k_d2f, nblocks(n), TPB, st, n, dst, src); }

void launch_add_f2d(cudaStream_t st, int n, double *dst, const float *src) { launch_k(k_add_f2d, nblocks(n), TPB, st, n, dst, src); }

void launch_residual64(cudaStream_t st, const Lvl &L, const double *K, const double *f, const double *u, double *r, Red red, double *out)
{
	launch_residual<double>(st, L, K, f, u, r);
	launch_k(k_dot, red_grid(L.neq), RED_THREADS, st, L.neq, (const double *)r, (const double *)r, red, out);
}

void launch_visc_from_T(cudaStream_t st, const Lvl &L, const Geo *geo, const Rheo &r, const double *T, double *evi)
{
	launch_k(k_visc_from_T, nblocks(L.nel), TPB, st, L, geo, r, T, evi);
}

void launch_strain_rate(cudaStream_t st, const Lvl &L, const Geo *geo, const double *V, double *edot)
{
	launch_k(k_strain_rate, nblocks(L.nel), TPB, st, L, geo, V, edot);
}

void launch_visc_from_S(cudaStream_t st, const Lvl &L, const Geo *geo, const Rheo &r, const double *T, const double *edot,
                        double *evi)
{
	launch_k(k_visc_from_S, nblocks(L.nel), TPB, st, L, geo, r, T, edot, evi);
}

void launch_project_viscosity(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, const Geo *geof, const Geo *geoc, const double *evi_f,
                              double *evi_c, double *work_f, double *work_c)
{
	launch_k(k_visc_to_nodes, nblocks(Lf.nno), TPB, st, Lf, geof, evi_f, work_f);
	launch_k(k_project_scalar, nblocks(Lc.nno), TPB, st, Lf, Lc, geoc, work_f, work_c);
	launch_k(k_visc_to_gint, nblocks(Lc.nel), TPB, st, Lc, geoc, work_c, evi_c);
}

void launch_buoyancy(cudaStream_t st, const Lvl &L, const Geo *geo, double Ra, const double *T, double *buoy)
{
	// the layer means go into the tail of `buoy`'s companion buffer: buoy + nno (caller sizes it nno + noz)
	double *H = buoy + L.nno;
	launch_k(k_horiz_ave, L.noz, TPB, st, L, geo, Ra, T, H);
	launch_k(k_buoyancy, nblocks(L.nno), TPB, st, L, Ra, T, H, buoy);
}

void launch_horiz_ave(cudaStream_t st, const Lvl &L, const Geo *geo, const double *T, double *H)
{
	launch_k(k_horiz_ave, L.noz, TPB, st, L, geo, 1.0, T, H);
}

void launch_forces(cudaStream_t st, const Lvl &L, const Geo *geo, const double *buoy, double *F)
{
	if(L.sphere)
		launch_k(k_forces, nblocks(L.nno), TPB, st, L, geo, buoy, F);
	else
		launch_k(k_forces_box, nblocks(L.nno), TPB, st, L, geo, buoy, F);
}

void launch_v_from_vector(cudaStream_t st, const Lvl &L, const double *U, double *V)
{
	launch_k(k_v_from_vector, nblocks(L.nno), TPB, st, L, U, V);
}

void launch_pg_residual(cudaStream_t st, const Lvl &L, const Geo *geo, const double *T, const double *Tdot, const double *V, double Q0,
                        double *Eres)
{
	if(L.sphere)
		launch_k(k_pg_residual, nblocks(L.nel, 128), 128, st, L, geo, T, Tdot, V, Q0, Eres);
	else
		launch_k(k_pg_residual_box, nblocks(L.nel, 128), 128, st, L, geo, T, Tdot, V, Q0, Eres);
}

void launch_pg_gather(cudaStream_t st, const Lvl &L, const Geo *geo, const double *Eres, double *DTdot)
{
	launch_k(k_pg_gather, nblocks(L.nno), TPB, st, L, geo, Eres, DTdot);
}

void launch_predictor(cudaStream_t st, const Lvl &L, double *T, double *Tdot, double dt, double gamma)
{
	launch_k(k_predictor, nblocks(L.nno), TPB, st, L, T, Tdot, dt, gamma);
}

void launch_corrector(cudaStream_t st, const Lvl &L, double *T, double *Tdot, const double *DTdot, double dt, double gamma)
{
	launch_k(k_corrector, nblocks(L.nno), TPB, st, L, T, Tdot, DTdot, dt, gamma);
}

void launch_tmax(cudaStream_t st, int n, const double *T, Red red, double *out)
{
	launch_k(k_max, red_grid(n), RED_THREADS, st, n, T, red, out);
}

void launch_adv_timestep(cudaStream_t st, const Lvl &L, const Geo *geo, const double *V, Red red, double *out)
{
	launch_k(k_adv_step, red_grid(L.nel), RED_THREADS, st, L, geo, V, red, out);
}

void launch_conform_T(cudaStream_t st, const Lvl &L, double *T) { launch_k(k_conform_T, nblocks(L.nno), TPB, st, L, T); }

void launch_heat_flux(cudaStream_t st, const Lvl &L, const Geo *geo, const double *T, const double *V, double *work, Red red, double *out)
{
	// work holds nel element means then nno nodal fluxes
	launch_k(k_hf_elem, nblocks(L.nel), TPB, st, L, geo, T, V, work);
	launch_k(k_hf_node, nblocks(L.nno), TPB, st, L, geo, work, work + L.nel);
	launch_k(k_hf_surface, red_grid((long)L.elx * L.ely), RED_THREADS, st, L, geo, work + L.nel, red, out);
}

void launch_vrms(cudaStream_t st, const Lvl &L, const Geo *geo, const double *V, Red red, double *out)
{
	launch_k(k_vrms, red_grid(L.nel), RED_THREADS, st, L, geo, V, red, out);
}

void launch_output_fields(cudaStream_t st, const Lvl &L, const Geo *geo, const double *T, const double *V, const double *evi, Red red,
                          double *f, double *scratch, double *ue, double *H, double *surf, double *sums, double *scal)
{
	const int noz = L.noz;
	// heat_flux: Have.T first (the element integrals need it), then the three
	// nodal fields, Nu from the unreplaced heatflux, the surface replacement and
	// the layer means Have.Rho / F / f
	launch_k(k_horiz_ave, noz, TPB, st, L, geo, 1.0, T, H);
	launch_k(k_out_elem, nblocks(L.nel), TPB, st, L, geo, T, V, (const double *)H, ue);
	launch_k(k_out_node, nblocks(L.nno), TPB, st, L, geo, (const double *)ue, f);
	launch_k(k_hf_surface, red_grid((long)L.elx * L.ely), RED_THREADS, st, L, geo, (const double *)f, red, sums);
	launch_k(k_out_surface, nblocks(L.nox * L.noy), TPB, st, L, f, surf);
	launch_k(k_horiz_ave, noz, TPB, st, L, geo, 1.0, (const double *)f, H + 3 * noz);
	launch_k(k_horiz_ave, noz, TPB, st, L, geo, 1.0, (const double *)(f + L.nno), H + 4 * noz);
	launch_k(k_horiz_ave, noz, TPB, st, L, geo, 1.0, (const double *)(f + 2 * (size_t)L.nno), H + 5 * noz);
	// averages: Have.vrms and Have.Vi, and the global Vrms
	launch_k(k_out_speed2, nblocks(L.nno), TPB, st, L, V, scratch);
	launch_k(k_horiz_ave, noz, TPB, st, L, geo, 1.0, (const double *)scratch, H + noz);
	launch_k(k_visc_to_nodes, nblocks(L.nno), TPB, st, L, geo, evi, scratch);
	launch_k(k_horiz_ave, noz, TPB, st, L, geo, 1.0, (const double *)scratch, H + 2 * noz);
	launch_k(k_vrms, red_grid(L.nel), RED_THREADS, st, L, geo, V, red, sums + 4);
	launch_k(k_out_final, nblocks(noz), TPB, st, L, (const double *)sums, scal, H);
}
