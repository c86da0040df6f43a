// Stencil kernels of the large levels (K u, residual, one Gauss-Seidel
// colour) on the tile-major stencil (level.h: tiles of 32 positions of one
// colour, 243 * 32 words each).
//
// These kernels are bound by HBM bandwidth: a colour sweep of the finest
// FP32 level streams 38 MB of stencil and reuses the L2-resident vector.  The
// CTAs are persistent; each walks its tiles (blockIdx.x, + gridDim.x, ...) and
// keeps S of them in flight: one thread issues a bulk copy (cp.async.bulk,
// the TMA engine, no registers) of a whole tile into a shared-memory stage
// and arms the stage's transaction barrier, so a tile's 31 KB (FP32) or 62 KB
// (FP64) arrive while the CTA computes on the stage before.  A CTA is nine
// warps: warp g takes the column of three slots (dx, dy) = (g % 3 - 1,
// g / 3 - 1), dz = -1, 0, 1, for the 32 nodes of the tile (lane = node), so
// a lane reads its node's three neighbours in that column (loaded one tile
// ahead, overlapping the copy), multiplies them by 27 stencil words of the
// stage (lane-consecutive, conflict-free) and leaves three partial rows in
// shared memory; the owner threads of (node, row) add the nine partials in
// column order and update.  Few instructions per node, so the copy engine and
// HBM set the pace.  Waits are bounded: a stage that does not arrive sets an
// error word, no further copy is issued, and the CTA waits (bounded) for the
// copies it has in flight before it leaves.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"

namespace {

#include "device.cuh"

constexpr int TB = CG_TILE;  // nodes per tile = lanes of a warp
constexpr int TT = 9 * 32;   // threads: nine warps, one per column of three slots
static_assert(TB == 32, "one lane per node of a tile");
template <typename T> struct TileCfg
{
	static constexpr int STAGES = sizeof(T) == 4 ? 3 : 2;
	static constexpr int MIN_CTAS = sizeof(T) == 4 ? 2 : 1;  // per SM
	static constexpr unsigned BYTES = CG_TILE_WORDS * sizeof(T);
	static constexpr size_t SMEM = (size_t)STAGES * CG_TILE_WORDS * sizeof(T) + 2 * 27 * TB * sizeof(T);
};

enum
{
	TK_GS = 0,   // out = d: one Gauss-Seidel colour
	TK_KU = 1,   // out = K u
	TK_RES = 2   // out = f - K u
};

__device__ __forceinline__ unsigned t_smem(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void t_issue(unsigned bar, unsigned dst, const void *src, unsigned bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst), "l"(src),
	             "r"(bytes), "r"(bar)
	             : "memory");
}

// the same copy with an L2 eviction priority (a createpolicy word)
__device__ __forceinline__ void t_issue_hint(unsigned bar, unsigned dst, const void *src, unsigned bytes,
                                             unsigned long long pol)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(dst),
	             "l"(src), "r"(bytes), "r"(bar), "l"(pol)
	             : "memory");
}

__device__ __forceinline__ unsigned long long t_policy_last()
{
	unsigned long long p;
	asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
	return p;
}

__device__ __forceinline__ unsigned long long t_policy_first()
{
	unsigned long long p;
	asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
	return p;
}

// the L2 priority of the stencil copy of `tile` (level.h: l2hint, l2keep)
__device__ __forceinline__ unsigned long long t_tile_policy(const Lvl &L, int tile, unsigned long long last,
                                                            unsigned long long first)
{
	int c = 0;
#pragma unroll
	for(int m = 1; m < 8; ++m)
		c += (tile >= L.toff[m]);
	const int n = L.toff[c + 1] - L.toff[c];
	return 1000LL * (tile - L.toff[c]) < (long long)L.l2keep * n ? last : first;
}

// bounded wait (about a second at most) for the phase of `bar` with this parity
__device__ __forceinline__ bool t_wait(unsigned bar, unsigned parity)
{
	for(int it = 0; it < (1 << 17); ++it)
	{
		unsigned ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(ok)
		             : "r"(bar), "r"(parity), "r"(10000u)
		             : "memory");
		if(ok)
			return true;
	}
	return false;
}

__device__ double g_tile_err;  // 1 when a stage wait timed out
// Failure-path test hook: while nonzero, the next CTA to start takes it (an
// atomic exchange to zero) and arms its first stage without issuing the copy,
// so that the bounded wait on that stage runs out with no copy in flight.
__device__ int g_tile_hold;

// bounded wait for the copies a CTA still has in flight after a stage wait
// timed out.  These copies read stencil words that exist in global memory, so
// they complete within microseconds; the limit (about 16 s) only keeps the
// wait finite, and the CTA does not leave before it while a copy may still
// write into its shared memory.
__device__ __forceinline__ bool t_drain(unsigned bar, unsigned parity)
{
	for(int it = 0; it < 16; ++it)
		if(t_wait(bar, parity))
			return true;
	return false;
}

template <typename T, int KIND>
__global__ void __launch_bounds__(TT, TileCfg<T>::MIN_CTAS) k_tile(Lvl L, const T *__restrict__ K, const T *__restrict__ BI,
                                                                  const T *__restrict__ f, const T *u, T *out, int colour)
{
	constexpr int S = TileCfg<T>::STAGES;
	extern __shared__ __align__(128) unsigned char smem_raw[];
	T *stage = reinterpret_cast<T *>(smem_raw);
	T *part = stage + S * CG_TILE_WORDS;  // two buffers of 81 * TB partial rows
	__shared__ __align__(8) unsigned long long bar[S];
	const int t0 = KIND == TK_GS ? L.toff[colour] : 0;
	const int t1 = KIND == TK_GS ? L.toff[colour + 1] : L.toff[8];
	const int ntile = t1 - t0;
	const int nmine = (int)blockIdx.x < ntile ? (ntile - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
	const unsigned bar0 = t_smem(bar), st0 = t_smem(stage);
	unsigned long long pol_last = 0, pol_first = 0;
	if(L.l2hint && threadIdx.x == 0)
	{
		pol_last = t_policy_last();
		pol_first = t_policy_first();
	}
	auto issue = [&](int k) {
		const int b = k % S;
		const size_t tile = (size_t)t0 + blockIdx.x + (size_t)k * gridDim.x;
		if(L.l2hint)
			t_issue_hint(bar0 + 8 * b, st0 + b * TileCfg<T>::BYTES, K + tile * CG_TILE_WORDS, TileCfg<T>::BYTES,
			             t_tile_policy(L, (int)tile, pol_last, pol_first));
		else
			t_issue(bar0 + 8 * b, st0 + b * TileCfg<T>::BYTES, K + tile * CG_TILE_WORDS, TileCfg<T>::BYTES);
	};
	if(threadIdx.x == 0)
	{
		for(int b = 0; b < S; ++b)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8 * b) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();
	int issued = 0, held = -1;
	if(threadIdx.x == 0)
	{
		if(nmine > 0 && g_tile_hold != 0 && atomicExch(&g_tile_hold, 0) != 0)
		{
			// test hook: stage 0 expects its bytes, but no copy is issued
			asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar0), "r"(TileCfg<T>::BYTES)
			             : "memory");
			held = 0;
			issued = 1;
		}
		for(; issued < S && issued < nmine; ++issued)
			issue(issued);
	}
	// The stencil is written only by the assembly, long before any launch
	// here, so its first copies start before the wait on the preceding kernel
	// (under programmatic dependent launch they overlap that kernel's tail);
	// the vectors, which the preceding kernel may write, are read after it.
	pdl_begin();
	bool ok = true;
	const int ln = threadIdx.x & 31, g = threadIdx.x >> 5;
	const int dx = g % 3 - 1, dy = g / 3 - 1;
	const int oq = threadIdx.x / 3, oi = threadIdx.x % 3;  // owner (node, row), threadIdx.x < 3 * cnt
	// a tile's owner data and the lane's nine neighbour values, loaded one
	// tile ahead so that their latency overlaps the previous tile's work
	struct Pre
	{
		int cnt, on;
		T fi, bi, di;
		T uv[9];  // [dz + 1][component]
	};
	auto prefetch = [&](int k, Pre &q) {
		q.cnt = 0;
		if(k >= nmine)
			return;
		const int tile = t0 + blockIdx.x + k * gridDim.x;
		int cc = colour;
		if(KIND != TK_GS)
		{
			cc = 0;
#pragma unroll
			for(int m = 1; m < 8; ++m)
				cc += (tile >= L.toff[m]);
		}
		const int q0 = (tile - L.toff[cc]) * TB;
		q.cnt = min(TB, L.coff[cc + 1] - L.coff[cc] - q0);
		q.on = 0;
		q.fi = q.bi = q.di = 0;
		if((int)threadIdx.x < 3 * q.cnt)
		{
			int x, y, z;
			cg_decode(L, cc, q0 + oq, x, y, z);
			q.on = cg_node(L, x, y, z);
			if(KIND != TK_KU)
				q.fi = f[3 * q.on + oi];
			if(KIND == TK_GS)
			{
				q.bi = BI[3 * (size_t)(L.coff[cc] + q0 + oq) + oi];
				q.di = u[3 * q.on + oi];
			}
		}
#pragma unroll
		for(int e = 0; e < 9; ++e)
			q.uv[e] = 0;
		if(ln < q.cnt)
		{
			int x, y, z;
			cg_decode(L, cc, q0 + ln, x, y, z);
			const int col = cg_node(L, clampi(x + dx, 0, L.nox - 1), clampi(y + dy, 0, L.noy - 1), 0);
#pragma unroll
			for(int kz = 0; kz < 3; ++kz)
			{
				// missing neighbours are clamped onto the node: their stencil block is zero
				const int m = col + clampi(z + kz - 1, 0, L.noz - 1);
				q.uv[3 * kz] = u[3 * m];
				q.uv[3 * kz + 1] = u[3 * m + 1];
				q.uv[3 * kz + 2] = u[3 * m + 2];
			}
		}
	};
	Pre cur;
	prefetch(0, cur);
	for(int k = 0; k < nmine; ++k)
	{
		const int b = k % S;
		if(ok)
			ok = t_wait(bar0 + 8 * b, (unsigned)((k / S) & 1));
		T *pb = part + (k & 1) * 27 * TB;
		const int cnt = cur.cnt;
		if(ln < cnt)
		{
			// slots 3g .. 3g+2 (dz = -1, 0, 1): word ((3s + j) * TB + ln) * 3 + i of the stage
			const T *ks = stage + (size_t)b * CG_TILE_WORDS + (9 * g * TB + ln) * 3;
			T a0 = 0, a1 = 0, a2 = 0;
#pragma unroll
			for(int kz = 0; kz < 3; ++kz)
#pragma unroll
				for(int j = 0; j < 3; ++j)
				{
					const T *kw = ks + (3 * kz + j) * TB * 3;
					const T uj = cur.uv[3 * kz + j];
					a0 += kw[0] * uj;
					a1 += kw[1] * uj;
					a2 += kw[2] * uj;
				}
			pb[(g * 3 + 0) * TB + ln] = a0;
			pb[(g * 3 + 1) * TB + ln] = a1;
			pb[(g * 3 + 2) * TB + ln] = a2;
		}
		const int on = cur.on;
		const T fi = cur.fi, bi = cur.bi, di = cur.di;
		// a Gauss-Seidel colour never reads values of its own colour, so the
		// next tile's loads may start before this tile's updates land
		prefetch(k + 1, cur);
		__syncthreads();  // stage b read by every thread; partials complete
		if(threadIdx.x == 0 && ok && issued < nmine)
		{
			// the threads' reads of stage b are ordered before the copy that refills it
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
			issue(issued++);
		}
		if((int)threadIdx.x < 3 * cnt)
		{
			T r = 0;
#pragma unroll
			for(int gg = 0; gg < 9; ++gg)
				r += pb[(gg * 3 + oi) * TB + oq];
			if(KIND == TK_GS)
				out[3 * on + oi] = di + (fi - r) * bi;
			else if(KIND == TK_KU)
				out[3 * on + oi] = r;
			else
				out[3 * on + oi] = fi - r;
		}
	}
	if(!ok)
	{
		g_tile_err = 1.0;
		// No copy was issued after the first wait that ran out.  Thread 0
		// issued every earlier one: those still in flight land before the CTA
		// leaves (a held stage has none).
		if(threadIdx.x == 0)
			for(int k = max(0, issued - S); k < issued; ++k)
				if(k != held)
					t_drain(bar0 + 8 * (k % S), (unsigned)((k / S) & 1));
	}
}

// The finest level's FP64 operator held as two FP32 stencils of the same
// layout, K = Kh + Kl (Kh the FP32 stencil the smoother uses, Kl the
// remainder), applied to FP64 vectors in double-float arithmetic: each
// product (Kh + Kl)(uh + ul) keeps its rounding error (an FMA recovers it)
// and the sums use Knuth's two-sum, about 46 significant bits per row.  The
// same bytes as the FP64 stencil, FP32 instructions instead of GB300's slow
// FP64 ones.  Structure as k_tile: persistent CTAs, nine warps, a stage per
// tile holding its Kh and Kl words (two bulk copies on one barrier).
constexpr int SP_STAGES = 2;
constexpr unsigned SP_BYTES = CG_TILE_WORDS * sizeof(float);
constexpr size_t SP_SMEM = (size_t)SP_STAGES * 2 * CG_TILE_WORDS * sizeof(float) + 2 * 27 * TB * sizeof(float2);

// (sh, sl) += (ah + al) (bh + bl), dropping al bl (two-product and two-sum)
__device__ __forceinline__ void sp_madd(float &sh, float &sl, float ah, float al, float bh, float bl)
{
	const float p = __fmul_rn(ah, bh);
	const float e = __fmaf_rn(ah, bh, -p);
	const float pl = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, e));
	const float t = __fadd_rn(sh, p);
	const float bp = __fsub_rn(t, sh);
	const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
	sh = t;
	sl = __fadd_rn(sl, __fadd_rn(err, pl));
}

// u (FP64) as FP32 pairs (hi, lo), once per product, so that the stencil
// kernel below does no FP64 work per neighbour
__global__ void k_split_vec(int n, const double *__restrict__ u, float2 *__restrict__ uv)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
	{
		const double v = u[i];
		const float h = (float)v;
		uv[i] = make_float2(h, (float)(v - (double)h));
	}
}

template <int KIND>
__global__ void __launch_bounds__(TT, 1) k_tile_split(Lvl L, const float *__restrict__ Kh, const float *__restrict__ Kl,
                                                     const double *__restrict__ f, const float2 *uv, double *out)
{
	constexpr int S = SP_STAGES;
	extern __shared__ __align__(128) unsigned char smem_raw[];
	float *stage = reinterpret_cast<float *>(smem_raw);  // [stage][hi, lo][CG_TILE_WORDS]
	float2 *part = reinterpret_cast<float2 *>(stage + S * 2 * CG_TILE_WORDS);  // partial rows as pairs
	__shared__ __align__(8) unsigned long long bar[S];
	const int ntile = L.toff[8];
	const int nmine = (int)blockIdx.x < ntile ? (ntile - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
	const unsigned bar0 = t_smem(bar), st0 = t_smem(stage);
	unsigned long long pol_last = 0, pol_first = 0;
	if(L.l2hint && threadIdx.x == 0)
	{
		pol_last = t_policy_last();
		pol_first = t_policy_first();
	}
	auto issue = [&](int k) {
		const int b = k % S;
		const size_t tile = (size_t)blockIdx.x + (size_t)k * gridDim.x;
		const unsigned bb = bar0 + 8 * b, dst = st0 + b * 2 * SP_BYTES;
		asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bb), "r"(2 * SP_BYTES) : "memory");
		if(L.l2hint)
		{
			const unsigned long long pol = t_tile_policy(L, (int)tile, pol_last, pol_first);
			asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(dst),
			             "l"(Kh + tile * CG_TILE_WORDS), "r"(SP_BYTES), "r"(bb), "l"(pol)
			             : "memory");
			asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(dst + SP_BYTES),
			             "l"(Kl + tile * CG_TILE_WORDS), "r"(SP_BYTES), "r"(bb), "l"(pol)
			             : "memory");
			return;
		}
		asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
		             "l"(Kh + tile * CG_TILE_WORDS), "r"(SP_BYTES), "r"(bb)
		             : "memory");
		asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst + SP_BYTES),
		             "l"(Kl + tile * CG_TILE_WORDS), "r"(SP_BYTES), "r"(bb)
		             : "memory");
	};
	if(threadIdx.x == 0)
	{
		for(int b = 0; b < S; ++b)
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8 * b) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();
	int issued = 0;
	if(threadIdx.x == 0)
		for(; issued < S && issued < nmine; ++issued)
			issue(issued);
	// the stencil is written only by the assembly, long before any launch
	// here; the vectors are read after the wait on the preceding kernel
	pdl_begin();
	bool ok = true;
	const int ln = threadIdx.x & 31, g = threadIdx.x >> 5;
	const int dx = g % 3 - 1, dy = g / 3 - 1;
	const int oq = threadIdx.x / 3, oi = threadIdx.x % 3;
	struct Pre
	{
		int cnt, on;
		double fi;
		float uh[9], ul[9];  // [dz + 1][component], u = uh + ul
	};
	auto prefetch = [&](int k, Pre &q) {
		q.cnt = 0;
		if(k >= nmine)
			return;
		const int tile = blockIdx.x + k * gridDim.x;
		int cc = 0;
#pragma unroll
		for(int m = 1; m < 8; ++m)
			cc += (tile >= L.toff[m]);
		const int q0 = (tile - L.toff[cc]) * TB;
		q.cnt = min(TB, L.coff[cc + 1] - L.coff[cc] - q0);
		q.on = 0;
		q.fi = 0.0;
		if((int)threadIdx.x < 3 * q.cnt)
		{
			int x, y, z;
			cg_decode(L, cc, q0 + oq, x, y, z);
			q.on = cg_node(L, x, y, z);
			if(KIND == TK_RES)
				q.fi = f[3 * q.on + oi];
		}
#pragma unroll
		for(int e = 0; e < 9; ++e)
			q.uh[e] = q.ul[e] = 0.f;
		if(ln < q.cnt)
		{
			int x, y, z;
			cg_decode(L, cc, q0 + ln, x, y, z);
			const int col = cg_node(L, clampi(x + dx, 0, L.nox - 1), clampi(y + dy, 0, L.noy - 1), 0);
#pragma unroll
			for(int kz = 0; kz < 3; ++kz)
			{
				// missing neighbours are clamped onto the node: their stencil block is zero
				const int m = col + clampi(z + kz - 1, 0, L.noz - 1);
#pragma unroll
				for(int c = 0; c < 3; ++c)
				{
					const float2 v = uv[3 * m + c];
					q.uh[3 * kz + c] = v.x;
					q.ul[3 * kz + c] = v.y;
				}
			}
		}
	};
	Pre cur;
	prefetch(0, cur);
	for(int k = 0; k < nmine; ++k)
	{
		const int b = k % S;
		if(ok)
			ok = t_wait(bar0 + 8 * b, (unsigned)((k / S) & 1));
		float2 *pb = part + (k & 1) * 27 * TB;
		const int cnt = cur.cnt;
		if(ln < cnt)
		{
			const float *kh = stage + (size_t)b * 2 * CG_TILE_WORDS + (9 * g * TB + ln) * 3;
			const float *kl = kh + CG_TILE_WORDS;
			float ah[3] = {0.f, 0.f, 0.f}, al[3] = {0.f, 0.f, 0.f};
#pragma unroll
			for(int kz = 0; kz < 3; ++kz)
#pragma unroll
				for(int j = 0; j < 3; ++j)
				{
					const int w = (3 * kz + j) * TB * 3;
#pragma unroll
					for(int i = 0; i < 3; ++i)
						sp_madd(ah[i], al[i], kh[w + i], kl[w + i], cur.uh[3 * kz + j], cur.ul[3 * kz + j]);
				}
#pragma unroll
			for(int i = 0; i < 3; ++i)
				pb[(g * 3 + i) * TB + ln] = make_float2(ah[i], al[i]);
		}
		const int on = cur.on;
		const double fi = cur.fi;
		prefetch(k + 1, cur);
		__syncthreads();  // stage b read by every thread; partials complete
		if(threadIdx.x == 0 && ok && issued < nmine)
		{
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
			issue(issued++);
		}
		if((int)threadIdx.x < 3 * cnt)
		{
			// the nine partial rows, in column order, as a pair; one FP64 sum at the end
			float rh = 0.f, rl = 0.f;
#pragma unroll
			for(int gg = 0; gg < 9; ++gg)
			{
				const float2 v = pb[(gg * 3 + oi) * TB + oq];
				const float t = __fadd_rn(rh, v.x), bp = __fsub_rn(t, rh);
				rl = __fadd_rn(rl, __fadd_rn(__fadd_rn(__fsub_rn(rh, __fsub_rn(t, bp)), __fsub_rn(v.x, bp)), v.y));
				rh = t;
			}
			const double r = (double)rh + (double)rl;
			out[3 * on + oi] = KIND == TK_KU ? r : fi - r;
		}
	}
	if(!ok)
	{
		g_tile_err = 1.0;
		// no copy was issued after the wait that ran out; the earlier ones
		// land before the CTA leaves
		if(threadIdx.x == 0)
			for(int k = max(0, issued - S); k < issued; ++k)
				t_drain(bar0 + 8 * (k % S), (unsigned)((k / S) & 1));
	}
}

int g_split_ctas = 0;

template <typename T> struct TileGrid
{
	static int ctas;  // persistent CTAs: SMs x resident CTAs per SM
};
template <typename T> int TileGrid<T>::ctas = 0;

template <typename T> int tile_init_t(int sms)
{
	const int smem = (int)TileCfg<T>::SMEM;
	cudaError_t e = cudaSuccess;
	int occ = 0;
	for(auto fn : {k_tile<T, TK_GS>, k_tile<T, TK_KU>, k_tile<T, TK_RES>})
	{
		if(e == cudaSuccess)
			e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
		int o = 0;
		if(e == cudaSuccess)
			e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, TT, smem);
		occ = occ ? std::min(occ, o) : o;
	}
	if(e != cudaSuccess || occ < 1)
		return -1;
	TileGrid<T>::ctas = sms * occ;
	return 0;
}

template <typename T, int KIND>
void launch_tile(cudaStream_t st, const Lvl &L, const T *K, const T *BI, const T *f, const T *u, T *out, int colour)
{
	const int ntile = KIND == TK_GS ? L.toff[colour + 1] - L.toff[colour] : L.toff[8];
	if(ntile <= 0)
		return;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(std::min(ntile, std::max(1, TileGrid<T>::ctas)));
	cfg.blockDim = dim3(TT);
	cfg.dynamicSmemBytes = TileCfg<T>::SMEM;
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = g_use_pdl ? 1 : 0;
	cudaLaunchKernelEx(&cfg, k_tile<T, KIND>, L, K, BI, f, u, out, colour);
	++g_kernel_launches;
}

} // namespace

int tile_init()
{
	int dev = 0, sms = 0;
	if(cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
		return -1;
	if(tile_init_t<float>(sms) != 0 || tile_init_t<double>(sms) != 0)
		return -1;
	int occ = 0;
	for(auto fn : {k_tile_split<TK_KU>, k_tile_split<TK_RES>})
	{
		int o = 0;
		if(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SP_SMEM) != cudaSuccess ||
		   cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, TT, SP_SMEM) != cudaSuccess || o < 1)
			return -1;
		occ = occ ? std::min(occ, o) : o;
	}
	g_split_ctas = sms * occ;
	return 0;
}

int tile_error_async(double *host, cudaStream_t st)
{
	return cudaMemcpyFromSymbolAsync(host, g_tile_err, sizeof(double), 0, cudaMemcpyDeviceToHost, st) == cudaSuccess ? 0 : -1;
}

int tile_error_reset_async(cudaStream_t st)
{
	static const double zero = 0.0;
	return cudaMemcpyToSymbolAsync(g_tile_err, &zero, sizeof(double), 0, cudaMemcpyHostToDevice, st) == cudaSuccess ? 0 : -1;
}

int tile_hold_next_copy()
{
	const int one = 1;
	return cudaMemcpyToSymbol(g_tile_hold, &one, sizeof(int)) == cudaSuccess ? 0 : -1;
}

template <typename T> void launch_tile_gs(cudaStream_t st, const Lvl &L, const T *K, const T *BI, const T *F, T *d, int colour)
{
	launch_tile<T, TK_GS>(st, L, K, BI, F, d, d, colour);
}

template <typename T> void launch_tile_kmul(cudaStream_t st, const Lvl &L, const T *K, const T *u, T *out)
{
	launch_tile<T, TK_KU>(st, L, K, (const T *)nullptr, (const T *)nullptr, u, out, 0);
}

template <typename T> void launch_tile_residual(cudaStream_t st, const Lvl &L, const T *K, const T *f, const T *u, T *out)
{
	launch_tile<T, TK_RES>(st, L, K, (const T *)nullptr, f, u, out, 0);
}

#define TILE_INST(T)                                                                                         \
	template void launch_tile_gs<T>(cudaStream_t, const Lvl &, const T *, const T *, const T *, T *, int);   \
	template void launch_tile_kmul<T>(cudaStream_t, const Lvl &, const T *, const T *, T *);                 \
	template void launch_tile_residual<T>(cudaStream_t, const Lvl &, const T *, const T *, const T *, T *);
TILE_INST(float)
TILE_INST(double)

void launch_tile_split(cudaStream_t st, const Lvl &L, const float *Kh, const float *Kl, const double *f, const double *u,
                       float2 *uv, double *out)
{
	const int ntile = L.toff[8];
	if(ntile <= 0)
		return;
	{
		cudaLaunchConfig_t c = {};
		c.gridDim = dim3((L.neq + 255) / 256);
		c.blockDim = dim3(256);
		c.stream = st;
		cudaLaunchAttribute a[1];
		a[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
		a[0].val.programmaticStreamSerializationAllowed = 1;
		c.attrs = a;
		c.numAttrs = g_use_pdl ? 1 : 0;
		cudaLaunchKernelEx(&c, k_split_vec, L.neq, u, uv);
		++g_kernel_launches;
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(std::min(ntile, std::max(1, g_split_ctas)));
	cfg.blockDim = dim3(TT);
	cfg.dynamicSmemBytes = SP_SMEM;
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = g_use_pdl ? 1 : 0;
	if(f)
		cudaLaunchKernelEx(&cfg, k_tile_split<TK_RES>, L, Kh, Kl, f, (const float2 *)uv, out);
	else
		cudaLaunchKernelEx(&cfg, k_tile_split<TK_KU>, L, Kh, Kl, f, (const float2 *)uv, out);
	++g_kernel_launches;
}
