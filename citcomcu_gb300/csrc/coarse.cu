// The coarse levels of one FP32 multigrid pass in one thread-block cluster.
//
// Below a few thousand nodes a level's Gauss-Seidel colour is too small to
// fill the GPU: a launch per colour costs its latency (launch, ramp, drain)
// however little it does.  The work of multi_grid (General_matrix_functions.c
// :525-653) at the levels 0..LC (smoothing, residual, projection,
// interpolation, line search and update) therefore runs as a short program of
// operations inside ONE cluster of up to 16 CTAs (one per SM), with cluster
// barriers where the reference's order needs them:
//  * Gauss-Seidel (gauss_seidel, General_matrix_functions.c:1160-1361, in 8
//    colours): every CTA keeps the whole correction vector of the level in
//    shared memory on a grid with a one-node zero halo, relaxes its share of
//    each colour's nodes (nine lanes per node, the padded stencil streamed
//    from L2 one colour ahead into registers), and stores each new node value
//    into every CTA's copy through distributed shared memory; one cluster
//    barrier per colour.  The coarsest level is relaxed by one CTA alone with
//    its stencil staged in shared memory and a CTA barrier per colour.
//  * residual / K u (n_assemble_del2_u, Element_calculations.c:552), the line
//    search dot products (FP64, fixed order: per-CTA partials exchanged through
//    distributed shared memory and summed in rank order by every CTA),
//    projection and interpolation (Solver_multigrid.c:72-298) split the nodes
//    of a level evenly over the CTAs.
// Every operation ends with a cluster barrier; data written by another CTA is
// read with L2 loads (ld.global.cg).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "kernels.h"

namespace cgp = cooperative_groups;

namespace {

#include "device.cuh"

constexpr int CO_THREADS = 512;
constexpr int CO_WARPS = CO_THREADS / 32;
constexpr int CO_NODES = 3 * CO_WARPS;  // nodes one pass of the CTA's warps relaxes
constexpr int CO_MAX_CLUSTER = 16;

__device__ __forceinline__ void co_chunk(int n, int rank, int ncta, int &lo, int &cnt)
{
	lo = n * rank / ncta;
	cnt = n * (rank + 1) / ncta - lo;
}

__device__ __forceinline__ int co_halo(const Lvl &L, int x, int y, int z)
{
	return (z + 1) + (L.noz + 2) * ((x + 1) + (L.nox + 2) * (y + 1));
}

// ---- distributed shared memory with transaction-counted barriers
__device__ __forceinline__ unsigned co_smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned co_mapa(unsigned addr, int rank)
{
	unsigned r;
	asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
	return r;
}

// 16 bytes into another CTA's shared memory; the write completes on that
// CTA's barrier as 16 bytes of transaction count
__device__ __forceinline__ void co_st_async(unsigned raddr, float4 v, unsigned rbar)
{
	asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(raddr), "f"(v.x),
	             "f"(v.y), "f"(v.z), "f"(v.w), "r"(rbar)
	             : "memory");
}

__device__ __forceinline__ void co_mbar_init(unsigned bar)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void co_mbar_expect(unsigned bar, unsigned bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool co_mbar_test(unsigned bar, unsigned parity)
{
	unsigned ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
	             : "=r"(ok)
	             : "r"(bar), "r"(parity)
	             : "memory");
	return ok != 0;
}

// suspends the thread until the phase completes or about `ns` pass
__device__ __forceinline__ bool co_mbar_try(unsigned bar, unsigned parity, unsigned ns)
{
	unsigned ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
	             : "=r"(ok)
	             : "r"(bar), "r"(parity), "r"(ns)
	             : "memory");
	return ok != 0;
}

// bounded wait (about a second at most) for the phase of `bar` with this
// parity; on time-out the error word is set and false returned (the caller
// then stops arming and storing: an arrival on a barrier whose phase is
// still open is not allowed)
#ifndef CO_SPIN
#define CO_SPIN 0
#endif
constexpr long CO_WAIT_LIMIT = CO_SPIN ? (1L << 24) : (1L << 17);
__device__ __forceinline__ bool co_mbar_wait(unsigned bar, unsigned parity, double *err)
{
	long it = 0;
	while(!(CO_SPIN ? co_mbar_test(bar, parity) : co_mbar_try(bar, parity, 10000u)))
		if(++it > CO_WAIT_LIMIT)
		{
			*err = 1.0;
			return false;
		}
	return true;
}

// a vector (written by other CTAs) into this CTA's shared memory, eight
// loads in flight per thread; ends with a CTA barrier.  Not inlined: its
// registers would otherwise weigh on the allocation of the smoother loop.
__device__ __noinline__ void co_stage(const float *v, int n, float *s)
{
	for(int b = threadIdx.x; b < n; b += 8 * blockDim.x)
	{
		float x[8];
#pragma unroll
		for(int k = 0; k < 8; ++k)
			if(b + k * (int)blockDim.x < n)
				x[k] = __ldcg(v + b + k * blockDim.x);
#pragma unroll
		for(int k = 0; k < 8; ++k)
			if(b + k * (int)blockDim.x < n)
				s[b + k * blockDim.x] = x[k];
	}
	__syncthreads();
}

// the level's vector d (node order) into the halo grid sd, zero halo; four
// cells (twelve loads) in flight per thread.  Not inlined (as co_stage).
__device__ __noinline__ void co_fill_halo(const Lvl &L, const float *d, bool zero, float4 *sd)
{
	const int HZ = L.noz + 2, HX = L.nox + 2, HN = HZ * HX * (L.noy + 2);
	for(int b = threadIdx.x; b < HN; b += 4 * blockDim.x)
	{
		float4 v[4];
		int n[4];
#pragma unroll
		for(int k = 0; k < 4; ++k)
		{
			const int t = b + k * blockDim.x;
			const int hz = t % HZ, hx = (t / HZ) % HX, hy = t / (HZ * HX);
			n[k] = (!zero && t < HN && hz >= 1 && hz <= L.noz && hx >= 1 && hx <= L.nox && hy >= 1 && hy <= L.noy)
			           ? cg_node(L, hx - 1, hy - 1, hz - 1)
			           : -1;
		}
#pragma unroll
		for(int k = 0; k < 4; ++k)
			v[k] = n[k] >= 0 ? make_float4(__ldcg(d + 3 * n[k]), __ldcg(d + 3 * n[k] + 1), __ldcg(d + 3 * n[k] + 2), 0.f)
			                 : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
		for(int k = 0; k < 4; ++k)
			if(b + k * (int)blockDim.x < HN)
				sd[b + k * blockDim.x] = v[k];
	}
}

// Gauss-Seidel sweeps of one level.  LOCAL: CTA 0 alone, stencil staged in
// shared memory, a CTA barrier per colour.  Otherwise every CTA relaxes its
// chunk of each colour's nodes and stores each new value into every CTA's
// halo grid with st.async; the stores complete on the receiving CTA's
// transaction barrier (two, alternating by colour), on which its warps wait
// before the next colour: no cluster-wide barrier per colour.  A CTA can be at
// most one colour ahead of another, and the barrier of a colour only completes
// after every warp that reads this colour's neighbours has sent its values,
// so no value is overwritten before it is read.  Ends with d written back.
template <bool LOCAL>
__device__ void co_gs(cgp::cluster_group &cl, const Lvl &L, const float4 *Kt, const float *BI, float *d, const float *f, int cycles,
                      bool zero, int win, float4 *arena, unsigned long long *bars, double *err)
{
	const int rank = LOCAL ? 0 : (int)cl.block_rank();
	const int ncta = LOCAL ? 1 : (int)cl.num_blocks();
	const int HZ = L.noz + 2, HXZ = (L.nox + 2) * HZ, HN = HXZ * (L.noy + 2);
	float4 *sd = arena;
	float4 *sFB = arena + HN;                                  // (F, 1/diag) of node j of colour c at 2 (48c + j)
	int2 *sLoc = reinterpret_cast<int2 *>(sFB + 16 * CO_NODES);  // (halo index, position) of node j of colour c at 48c + j
	float4 *sK = reinterpret_cast<float4 *>(sLoc + 8 * CO_NODES);
	co_fill_halo(L, d, zero, sd);
	for(int t = threadIdx.x; t < 8 * CO_NODES; t += blockDim.x)
	{
		const int c = t / CO_NODES, q = t - CO_NODES * c;
		int lo, cnt;
		co_chunk(L.coff[c + 1] - L.coff[c], rank, ncta, lo, cnt);
		if(q >= cnt)
		{
			sLoc[t] = make_int2(-1, 0);
			continue;
		}
		int x, y, z;
		cg_decode(L, c, lo + q, x, y, z);
		const int n = cg_node(L, x, y, z), p = L.coff[c] + lo + q;
		sLoc[t] = make_int2(co_halo(L, x, y, z), p);
		sFB[2 * t] = make_float4(__ldcg(f + 3 * n), __ldcg(f + 3 * n + 1), __ldcg(f + 3 * n + 2), 0.f);
		sFB[2 * t + 1] = make_float4(__ldg(BI + 3 * p), __ldg(BI + 3 * p + 1), __ldg(BI + 3 * p + 2), 0.f);
	}
	const float4 *Kb = Kt;
	if(LOCAL)
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
		Kb = sK;
		__syncthreads();
	}
	else
	{
		if(threadIdx.x == 0)
		{
			co_mbar_init(co_smem_addr(bars));
			co_mbar_init(co_smem_addr(bars + 1));
			asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		}
		cl.sync();  // halo grids and barriers of every CTA ready before any store
	}
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int sub = lane / 9, r9 = lane - 9 * sub, j = 3 * warp + sub;
	const int uoff = -1 + HZ * (r9 % 3 - 1) + HXZ * (r9 / 3 - 1);
	const unsigned sd_a = co_smem_addr(sd), bar_a = co_smem_addr(bars);
	// a node's value goes to the CTAs within `win` ranks of its owner (they
	// hold all its neighbours): this lane stores to wlo + r9 and wlo + r9 + 9
	const int wlo = max(0, rank - win), whi = min(ncta - 1, rank + win);
	unsigned ra0 = 0xffffffffu, ra1 = 0xffffffffu;
	if(!LOCAL)
	{
		if(wlo + r9 <= whi)
			ra0 = (unsigned)(wlo + r9);
		if(wlo + r9 + 9 <= whi)
			ra1 = (unsigned)(wlo + r9 + 9);
	}
	const int nph = 8 * cycles;
	// stencil words of the lane's node of the current colour (prefetched one colour ahead)
	float4 kc[7];
	auto node_of = [&](int c, int &hp, int &p) {
		if(lane >= 27)
			return false;
		const int2 hl = sLoc[CO_NODES * c + j];
		hp = hl.x;
		p = hl.y;
		return hl.x >= 0;
	};
	int hp = 0, p = 0;
	bool act = node_of(0, hp, p);
	if(!LOCAL && act)
#pragma unroll
		for(int t = 0; t < 7; ++t)
			kc[t] = __ldg(Kb + (size_t)63 * p + 7 * r9 + t);
	unsigned uses0 = 0, uses1 = 0;  // completed phases of the two barriers
	bool ok = true;                 // false after a timed-out wait: no more arrivals or stores
	for(int ph = 0; ph < nph; ++ph)
	{
		const int c = ph & 7, b = ph & 1;
		if(!LOCAL && threadIdx.x == 0 && ok)
		{
			// the values of colour c owned by the ranks wlo .. whi
			const int nc = L.coff[c + 1] - L.coff[c];
			co_mbar_expect(bar_a + 8 * b, (unsigned)(16 * (nc * (whi + 1) / ncta - nc * wlo / ncta)));
		}
		float4 dv = make_float4(0.f, 0.f, 0.f, 0.f), fv = dv, bv = dv;
		float r0 = 0.f, r1 = 0.f, r2 = 0.f;
		if(act)
		{
			if(r9 == 0)
			{
				dv = sd[hp];
				fv = sFB[2 * (CO_NODES * c + j)];
				bv = sFB[2 * (CO_NODES * c + j) + 1];
			}
			kt_rows(LOCAL ? Kb + (size_t)63 * p + 7 * r9 : kc, sd + hp + uoff, r0, r1, r2);
		}
		const int hp_c = hp;
		const bool act_c = act;
		if(ph + 1 < nph)
		{
			act = node_of((ph + 1) & 7, hp, p);
			if(!LOCAL && act)
#pragma unroll
				for(int t = 0; t < 7; ++t)
					kc[t] = __ldg(Kb + (size_t)63 * p + 7 * r9 + t);
		}
		r0 = kt_sum9(r0, lane);
		r1 = kt_sum9(r1, lane);
		r2 = kt_sum9(r2, lane);
		if(act_c && r9 == 0)
		{
			dv.x += (fv.x - r0) * bv.x;
			dv.y += (fv.y - r1) * bv.y;
			dv.z += (fv.z - r2) * bv.z;
		}
		if(LOCAL)
		{
			if(act_c && r9 == 0)
				sd[hp_c] = dv;
			asm volatile("bar.sync 1, %0;" ::"r"(CO_THREADS) : "memory");
		}
		else
		{
			const int src = 9 * sub;
			dv.x = __shfl_sync(0xffffffffu, dv.x, src);
			dv.y = __shfl_sync(0xffffffffu, dv.y, src);
			dv.z = __shfl_sync(0xffffffffu, dv.z, src);
			if(act_c && ok)
			{
				const unsigned off = 16u * (unsigned)hp_c;
				if(ra0 != 0xffffffffu)
					co_st_async(co_mapa(sd_a + off, ra0), dv, co_mapa(bar_a + 8 * b, ra0));
				if(ra1 != 0xffffffffu)
					co_st_async(co_mapa(sd_a + off, ra1), dv, co_mapa(bar_a + 8 * b, ra1));
			}
			if(ok)
				ok = co_mbar_wait(bar_a + 8 * b, (b ? uses1 : uses0) & 1u, err);
			if(b)
				++uses1;
			else
				++uses0;
		}
	}
	if(!LOCAL)
		cl.sync();  // every CTA past its last wait before the barriers are re-armed by a later call
	// write back this CTA's nodes
	for(int t = threadIdx.x; t < 8 * CO_NODES; t += blockDim.x)
	{
		const int2 hl = sLoc[t];
		if(hl.x < 0)
			continue;
		int c, x, y, z;
		pos_xyz(L, hl.y, c, x, y, z);
		const int n = cg_node(L, x, y, z);
		const float4 v = sd[hl.x];
		d[3 * n] = v.x;
		d[3 * n + 1] = v.y;
		d[3 * n + 2] = v.z;
	}
}

// K u over this CTA's nodes (its chunk of every colour, as in the smoother,
// so that the halo values the smoother left are the ones needed here), u in
// the halo grid sd.  MODE 0 (residual): out = f - K u.  MODE 1 (line search):
// out = K u, and lane r9 == 0 of each node accumulates out.f and out.out
// (in FP32 over its few nodes; the lanes' partials are then added in FP64).
// The CTA's nodes are listed first (position, halo index, node index
// in sloc, their count in *stot), then taken 48 at a time (one pass on the
// small levels).
constexpr int CO_MAX_OWN = 8 * CO_NODES;

__device__ void co_list(const Lvl &L, int rank, int ncta, int4 *sloc, int *stot)
{
	__shared__ int pre[9], los[8];
	if(threadIdx.x == 0)
	{
		int acc = 0;
		for(int c = 0; c < 8; ++c)
		{
			int lo, cnt;
			co_chunk(L.coff[c + 1] - L.coff[c], rank, ncta, lo, cnt);
			pre[c] = acc;
			los[c] = lo;
			acc += cnt;
		}
		pre[8] = acc;
		*stot = acc;
	}
	__syncthreads();
	for(int t = threadIdx.x; t < pre[8]; t += blockDim.x)
	{
		int c = 0;
		for(int k = 1; k < 8; ++k)
			c += (t >= pre[k]);
		const int q = los[c] + t - pre[c];
		int x, y, z;
		cg_decode(L, c, q, x, y, z);
		sloc[t] = make_int4(L.coff[c] + q, co_halo(L, x, y, z), cg_node(L, x, y, z), 0);
	}
	__syncthreads();
}

template <int MODE>
__device__ void co_kmul(const Lvl &L, const float4 *Kt, const float4 *sd, const float *f, float *out, float &ab, float &aa,
                        const int4 *sloc, int tot)
{
	const int HZ = L.noz + 2, HXZ = (L.nox + 2) * HZ;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const int sub = lane / 9, r9 = lane - 9 * sub;
	const int uoff = -1 + HZ * (r9 % 3 - 1) + HXZ * (r9 / 3 - 1);
	for(int b = 0; b < tot; b += CO_NODES)
	{
		const int t = b + 3 * warp + sub;
		const bool act = lane < 27 && t < tot;
		float r0 = 0.f, r1 = 0.f, r2 = 0.f, f0 = 0.f, f1 = 0.f, f2 = 0.f;
		int n = 0;
		if(act)
		{
			const int4 e = sloc[t];
			n = e.z;
			if(r9 == 0)
			{
				f0 = __ldcg(f + 3 * n);
				f1 = __ldcg(f + 3 * n + 1);
				f2 = __ldcg(f + 3 * n + 2);
			}
			float4 k[7];
			const float4 *kr = Kt + (size_t)63 * e.x + 7 * r9;
#pragma unroll
			for(int u = 0; u < 7; ++u)
				k[u] = __ldg(kr + u);
			kt_rows(k, sd + e.y + uoff, r0, r1, r2);
		}
		r0 = kt_sum9(r0, lane);
		r1 = kt_sum9(r1, lane);
		r2 = kt_sum9(r2, lane);
		if(act && r9 == 0)
		{
			if(MODE == 0)
			{
				out[3 * n] = f0 - r0;
				out[3 * n + 1] = f1 - r1;
				out[3 * n + 2] = f2 - r2;
			}
			else
			{
				out[3 * n] = r0;
				out[3 * n + 1] = r1;
				out[3 * n + 2] = r2;
				ab += r0 * f0 + r1 * f1 + r2 * f2;
				aa += r0 * r0 + r1 * r1 + r2 * r2;
			}
		}
	}
}

// vel += alpha del over this CTA's nodes (listed by co_list)
__device__ void co_update(float *vel, const float *del, float alpha, const int4 *sloc, int tot)
{
	for(int t = threadIdx.x; t < tot; t += blockDim.x)
	{
		const int n = sloc[t].z;
		float v[3], e[3];
#pragma unroll
		for(int i = 0; i < 3; ++i)
		{
			v[i] = __ldcg(vel + 3 * n + i);
			e[i] = __ldcg(del + 3 * n + i);
		}
#pragma unroll
		for(int i = 0; i < 3; ++i)
			vel[3 * n + i] = v[i] + alpha * e[i];
	}
}

__global__ void __launch_bounds__(CO_THREADS) k_coarse(const __grid_constant__ CoLevels D, const __grid_constant__ CoProg P)
{
	pdl_begin();
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__shared__ double wsum[CO_WARPS][2];
	__shared__ double csum[CO_MAX_CLUSTER][2];  // per-CTA line-search partials, written by every CTA
	__shared__ __align__(8) unsigned long long bars[2];  // transaction barriers of the cluster smoother
	__shared__ int4 sloc[CO_MAX_OWN];                     // the CTA's nodes (co_list)
	__shared__ int stot;
	float4 *arena = reinterpret_cast<float4 *>(smem_raw);
	cgp::cluster_group cl = cgp::this_cluster();
	const int rank = (int)cl.block_rank(), ncta = (int)cl.num_blocks();
	int halo_lev = -1, halo_vec = -1;  // (level, vector) whose current values sit in every CTA's halo grid
	double alpha = 0.0;
	// the program's stencils were evicted from L2 by the finer levels' work:
	// each CTA asks for its share of every level's padded stencil at once
	if(threadIdx.x == 0)
		for(int l = 0; l < D.nlev; ++l)
		{
			const unsigned long long total = 16ull * 63ull * (unsigned long long)D.L[l].nno;
			const unsigned long long a = (total * rank / ncta) & ~15ull, b = (total * (rank + 1) / ncta) & ~15ull;
			const char *base = reinterpret_cast<const char *>(D.Kt[l]);
			for(unsigned long long o = a; o < b; o += 65536ull)
			{
				const unsigned sz = (unsigned)((b - o) < 65536ull ? (b - o) : 65536ull);
				asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(base + o), "r"(sz) : "memory");
			}
		}
	cl.sync();  // all CTAs of the cluster running before any distributed shared memory access
	for(int o = 0; o < P.n; ++o)
	{
		const CoOp op = P.op[o];
		const int l = op.lev;
		const Lvl &L = D.L[l];
		switch(op.type)
		{
		case CO_GS:
			if(op.local)
			{
				if(rank == 0)
					co_gs<true>(cl, L, D.Kt[l], D.BI[l], D.vec[l][op.a], D.vec[l][op.b], op.cycles, op.zero != 0, D.win[l], arena, bars, D.err);
				halo_lev = -1;
			}
			else
			{
				co_gs<false>(cl, L, D.Kt[l], D.BI[l], D.vec[l][op.a], D.vec[l][op.b], op.cycles, op.zero != 0, D.win[l], arena, bars, D.err);
				halo_lev = l;
				halo_vec = op.a;
			}
			break;
		case CO_RESID:
		case CO_KDOT:
		{
			// CO_RESID: vec c = vec a - K vec b;  CO_KDOT: vec c = K vec a, alpha = (c.b) / (c.c)
			const int uvec = op.type == CO_RESID ? op.b : op.a;
			if(halo_lev != l || halo_vec != uvec)
			{
				co_fill_halo(L, D.vec[l][uvec], false, arena);
				__syncthreads();
				halo_lev = l;
				halo_vec = uvec;
			}
			float abf = 0.f, aaf = 0.f;
			co_list(L, rank, ncta, sloc, &stot);
			if(op.type == CO_RESID)
				co_kmul<0>(L, D.Kt[l], arena, D.vec[l][op.a], D.vec[l][op.c], abf, aaf, sloc, stot);
			else
			{
				co_kmul<1>(L, D.Kt[l], arena, D.vec[l][op.b], D.vec[l][op.c], abf, aaf, sloc, stot);
				double ab = abf, aa = aaf;
				// fixed-order sums: lanes, warps, then CTAs in rank order
				for(int s = 16; s > 0; s >>= 1)
				{
					ab += __shfl_xor_sync(0xffffffffu, ab, s);
					aa += __shfl_xor_sync(0xffffffffu, aa, s);
				}
				if((threadIdx.x & 31) == 0)
				{
					wsum[threadIdx.x >> 5][0] = ab;
					wsum[threadIdx.x >> 5][1] = aa;
				}
				__syncthreads();
				if(threadIdx.x < (unsigned)ncta)
				{
					double s0 = 0.0, s1 = 0.0;
					for(int w = 0; w < CO_WARPS; ++w)
					{
						s0 += wsum[w][0];
						s1 += wsum[w][1];
					}
					double *dst = cl.map_shared_rank(&csum[0][0], (int)threadIdx.x);
					dst[2 * rank] = s0;
					dst[2 * rank + 1] = s1;
				}
				cl.sync();
				if(threadIdx.x == 0)
				{
					double s0 = 0.0, s1 = 0.0;
					for(int r = 0; r < ncta; ++r)
					{
						s0 += csum[r][0];
						s1 += csum[r][1];
					}
					wsum[0][0] = s0 / s1;  // one FP64 division, not one per thread
				}
				__syncthreads();
				alpha = wsum[0][0];
				if(op.zero)
				{
					// the update of the line search on the same nodes (vel += alpha del)
					co_update(D.vec[l][CO_VEL], D.vec[l][op.a], (float)alpha, sloc, stot);
					if(halo_lev == l && halo_vec == CO_VEL)
						halo_lev = -1;
				}
			}
			if(halo_lev == l && halo_vec == op.c)
				halo_lev = -1;
			break;
		}
		case CO_DENSE:
		{
			// vec a = N vec b (or += with a start): this CTA's rows, one warp
			// per row, the right-hand side staged in shared memory
			float *sv = reinterpret_cast<float *>(arena);
			const int n = L.neq;
			co_stage(D.vec[l][op.b], n, sv);
			int lo, cnt;
			co_chunk(n, rank, ncta, lo, cnt);
			const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
			float *out = D.vec[l][op.a];
			const float *Nl = D.dense[l];
			for(int i = lo + warp; i < lo + cnt; i += CO_WARPS)
			{
				const float *row = Nl + (size_t)i * n;
				float s = 0.f;
				for(int k = lane; k < n; k += 32)
					s += __ldg(row + k) * sv[k];
#pragma unroll
				for(int o = 16; o > 0; o >>= 1)
					s += __shfl_xor_sync(0xffffffffu, s, o);
				if(lane == 0)
					out[i] = op.zero ? s : __ldcg(out + i) + s;
			}
			halo_lev = -1;
			break;
		}
		case CO_UPD:
		{
			// vec a += alpha vec b (the level's line-search step)
			float *v = D.vec[l][op.a];
			const float *dl = D.vec[l][op.b];
			int lo, cnt;
			co_chunk(L.neq, rank, ncta, lo, cnt);
			for(int i = lo + threadIdx.x; i < lo + cnt; i += blockDim.x)
				v[i] = __ldcg(v + i) + (float)(alpha * (double)__ldcg(dl + i));
			if(halo_lev == l && halo_vec == op.a)
				halo_lev = -1;
			break;
		}
		case CO_PROJ:
		{
			// vec b of level l-1 = projection of vec a of level l, stripped
			// (the fine vector staged in shared memory, sums in FP32)
			const Lvl &Lc = D.L[l - 1];
			float *sv = reinterpret_cast<float *>(arena);
			co_stage(D.vec[l][op.a], L.neq, sv);
			int lo, cnt;
			co_chunk(Lc.nno, rank, ncta, lo, cnt);
			for(int b = 8 * lo; b < 8 * (lo + cnt); b += blockDim.x)
			{
				const int t = b + threadIdx.x;
				project_lanes<false, float, float>(L, Lc, D.geo[l - 1], sv, D.vec[l - 1][op.b], t < 8 * (lo + cnt) ? t : 8 * Lc.nno);
			}
			halo_lev = -1;
			break;
		}
		case CO_INTERP:
		{
			// vec b of level l = interpolation of vec a of level l-1, stripped
			// (the coarse vector staged in shared memory)
			float *sv = reinterpret_cast<float *>(arena);
			co_stage(D.vec[l - 1][op.a], D.L[l - 1].neq, sv);
			int lo, cnt;
			co_chunk(L.nno, rank, ncta, lo, cnt);
			for(int n = lo + threadIdx.x; n < lo + cnt; n += blockDim.x)
				if(L.sphere)
					interp_node<false, true, float>(D.L[l - 1], L, D.geo[l], sv, D.vec[l][op.b], n);
				else
					interp_node<false, false, float>(D.L[l - 1], L, D.geo[l], sv, D.vec[l][op.b], n);
			halo_lev = -1;
			break;
		}
		default:
			break;
		}
		cl.sync();
	}
}

// halo grid, (F, 1/diag) and location of up to 48 nodes per colour, [padded stencil]
size_t co_gs_bytes(const Lvl &L, bool local)
{
	const size_t hn = (size_t)(L.nox + 2) * (L.noy + 2) * (L.noz + 2);
	return 16 * (hn + 16 * CO_NODES) + 8 * 8 * CO_NODES + (local ? (size_t)16 * 63 * L.nno : 0);
}

// column j of the coarsest smoother's matrix: the one-CTA smoother of the
// cluster program run from d = 0 against f = e_j (work[j n ..] holds e_j,
// work[n^2 + j n ..] receives the column)
__global__ void __launch_bounds__(CO_THREADS) k_co_dense_build(Lvl L, const float4 *Kt, const float *BI, int cycles, float *work, double *err)
{
	pdl_begin();
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__shared__ __align__(8) unsigned long long bars[2];
	const int n = L.neq, j = blockIdx.x;
	float *f = work + (size_t)j * n;
	float *d = work + (size_t)n * n + (size_t)j * n;
	for(int i = threadIdx.x; i < n; i += blockDim.x)
		f[i] = (i == j) ? 1.f : 0.f;
	__threadfence();
	__syncthreads();
	cgp::cluster_group cl = cgp::this_cluster();
	co_gs<true>(cl, L, Kt, BI, d, f, cycles, true, 0, reinterpret_cast<float4 *>(smem_raw), bars, err);
}

// N[i][j] = column j, entry i
__global__ void k_co_dense_t(int n, const float *cols, float *N)
{
	pdl_begin();
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if(t >= n * n)
		return;
	const int i = t / n, j = t - i * n;
	N[t] = cols[(size_t)j * n + i];
}

// columns j0 .. j0+nb-1 of a level's smoother matrix: `cycles` zero-start
// sweeps of the 8 colours (each node of a colour: r = f - K d over its 27
// neighbours, then d += r o 1/diag, the update of gauss_seidel) against f =
// e_j; N[i n + j] = d_i.  The rows of a colour are formed before any of its
// nodes is updated (a node's own block reads its old values).  A CTA relaxes
// nb columns at once, their d in shared memory: the threads of one row and
// its nb columns are adjacent, so each stencil word is read from L2 once per
// CTA for all of them (one column per CTA read the level's stencil once per
// column).  Each entry keeps the per-column summation order.
__global__ void __launch_bounds__(256) k_dense_build_gs(Lvl L, const float *__restrict__ K, const float *__restrict__ BI,
                                                        int cycles, int ncols, int maxrows, float *N)
{
	pdl_begin();
	extern __shared__ __align__(16) float db_smem[];
	const int n = L.neq, j0 = blockIdx.x * ncols;
	const int nb = min(ncols, n - j0);
	float *d = db_smem;             // [b][n]
	float *rs = db_smem + ncols * n;  // [b][maxrows]
	for(int i = threadIdx.x; i < ncols * n; i += blockDim.x)
		d[i] = 0.f;
	__syncthreads();
	for(int cyc = 0; cyc < cycles; ++cyc)
		for(int c = 0; c < 8; ++c)
		{
			const int cnt = L.coff[c + 1] - L.coff[c];
			for(int t = threadIdx.x; t < 3 * cnt * nb; t += blockDim.x)
			{
				const int row = t / nb, b = t - nb * row;
				const int q = row / 3, i = row - 3 * q, p = L.coff[c] + q;
				int x, y, z;
				cg_decode(L, c, q, x, y, z);
				const float *db = d + (size_t)b * n;
				float r = (3 * cg_node(L, x, y, z) + i == j0 + b) ? 1.f : 0.f;
				for(int s = 0; s < 27; ++s)
				{
					const int mz = z + s % 3 - 1, mx = x + (s / 3) % 3 - 1, my = y + s / 9 - 1;
					if(mx < 0 || mx >= L.nox || my < 0 || my >= L.noy || mz < 0 || mz >= L.noz)
						continue;
					const int m = cg_node(L, mx, my, mz);
#pragma unroll
					for(int jj = 0; jj < 3; ++jj)
						r -= K[cg_kidx(L, s, i, jj, p)] * db[3 * m + jj];
				}
				rs[(size_t)b * maxrows + row] = r * BI[3 * (size_t)p + i];
			}
			__syncthreads();
			for(int t = threadIdx.x; t < 3 * cnt * nb; t += blockDim.x)
			{
				const int row = t / nb, b = t - nb * row;
				const int q = row / 3, i = row - 3 * q;
				int x, y, z;
				cg_decode(L, c, q, x, y, z);
				d[(size_t)b * n + 3 * cg_node(L, x, y, z) + i] += rs[(size_t)b * maxrows + row];
			}
			__syncthreads();
		}
	for(int t = threadIdx.x; t < n * nb; t += blockDim.x)
	{
		const int i = t / nb, b = t - nb * i;
		N[(size_t)i * n + j0 + b] = d[(size_t)b * n + i];
	}
}

} // namespace

void launch_dense_build_gs(cudaStream_t st, const Lvl &L, const float *K, const float *BI, int cycles, float *N)
{
	int maxc = 0;
	for(int c = 0; c < 8; ++c)
		maxc = std::max(maxc, L.coff[c + 1] - L.coff[c]);
	const int maxrows = 3 * maxc;
	// as many columns per CTA as fit in the shared memory the kernel may use
	const size_t per_col = sizeof(float) * (size_t)(L.neq + maxrows);
	const int ncols = (int)std::max<size_t>(1, std::min<size_t>(8, (size_t)CO_SMEM_MAX / per_col));
	const size_t smem = per_col * ncols;
	k_dense_build_gs<<<(L.neq + ncols - 1) / ncols, 256, smem, st>>>(L, K, BI, cycles, ncols, maxrows, N);
	++g_kernel_launches;
}

int coarse_init(int *cluster_size)
{
	*cluster_size = 0;
	if(cudaFuncSetAttribute(k_coarse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CO_SMEM_MAX) != cudaSuccess ||
	   cudaFuncSetAttribute(k_co_dense_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CO_SMEM_MAX) != cudaSuccess ||
	   cudaFuncSetAttribute(k_dense_build_gs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CO_SMEM_MAX) != cudaSuccess)
		return -1;
	cudaFuncSetAttribute(k_coarse, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
	for(int cs = CO_MAX_CLUSTER; cs >= 8; cs /= 2)
	{
		cudaLaunchConfig_t cfg = {};
		cfg.gridDim = dim3(cs);
		cfg.blockDim = dim3(CO_THREADS);
		cfg.dynamicSmemBytes = CO_SMEM_MAX;
		cudaLaunchAttribute attr[1];
		attr[0].id = cudaLaunchAttributeClusterDimension;
		attr[0].val.clusterDim.x = cs;
		attr[0].val.clusterDim.y = 1;
		attr[0].val.clusterDim.z = 1;
		cfg.attrs = attr;
		cfg.numAttrs = 1;
		int n = 0;
		if(cudaOccupancyMaxActiveClusters(&n, k_coarse, &cfg) == cudaSuccess && n > 0)
		{
			*cluster_size = cs;
			return 0;
		}
		cudaGetLastError();
	}
	return -1;
}

// whether level L can run in the cluster program, and whether its smoother
// runs on one CTA (local: the coarsest level, when it fits)
bool coarse_level_ok(const Lvl &L, int level, int cluster, bool *local)
{
	int maxc = 0;
	for(int c = 0; c < 8; ++c)
		maxc = std::max(maxc, L.coff[c + 1] - L.coff[c]);
	*local = level == 0 && maxc <= CO_NODES && co_gs_bytes(L, true) <= CO_SMEM_MAX;
	if(*local)
		return true;
	return (maxc + cluster - 1) / cluster <= CO_NODES && co_gs_bytes(L, false) <= CO_SMEM_MAX;
}

size_t coarse_smem(const Lvl &L, bool local) { return co_gs_bytes(L, local); }

int coarse_window(const Lvl &L, int cluster) { return cg_owner_window(L, cluster); }

void launch_coarse_dense_build(cudaStream_t st, const Lvl &L, const float4 *Kt, const float *BI, int cycles, float *work, float *N,
                               double *err)
{
	const int n = L.neq;
	k_co_dense_build<<<n, CO_THREADS, co_gs_bytes(L, true), st>>>(L, Kt, BI, cycles, work, err);
	k_co_dense_t<<<(n * n + 255) / 256, 256, 0, st>>>(n, work + (size_t)n * n, N);
	g_kernel_launches += 2;
}

void launch_coarse(cudaStream_t st, const CoLevels &D, const CoProg &P, int cluster, size_t smem)
{
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(cluster);
	cfg.blockDim = dim3(CO_THREADS);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = st;
	cudaLaunchAttribute attr[2];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = cluster;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[1].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = g_use_pdl ? 2 : 1;
	cudaLaunchKernelEx(&cfg, k_coarse, D, P);
	++g_kernel_launches;
}
