// Operator assembly of the box levels in double-float arithmetic (the mixed
// configuration).
//
// construct_node_ks (Construct_arrays.c:359-535) with get_elt_k / get_aug_k
// (Element_calculations.c:133-293, 1127-1163): every 3x3 block of a node's
// 27-block stencil row is the sum, over the (up to 8) elements holding both
// nodes, of sum_k eta_k Mk[k][a][b] plus the augmented term lambda mean(eta)
// g_a g_b^T.  k_assemble (kernels.cu) forms these sums in FP64, about 5,200
// FMA per node, and GB300's FP64 rate makes that the largest piece of a time
// step outside the multigrid passes.  Here every product and sum is carried
// as an unevaluated pair of FP32 numbers (hi + lo): the product of two pairs
// keeps its rounding error exactly (an FMA recovers it) and the sums use
// Knuth's two-sum, so an entry carries about 46 significant bits, of which
// the FP64 stencil keeps 46 and the FP32 stencil 24.  The FP64 pipe only
// converts the finished entries.
//
// With K32lo the entry's FP32 remainder (entry - K32) is written as well:
// the finest level's FP64 operator held as the pair K32 + K32lo (tile.cu,
// k_tile_split).
//
// Work split: one warp per (tile of 32 colour positions, slot); lane = node,
// so the nine words a lane writes per slot are consecutive with its
// neighbours' in the tile-major stencil (level.h, cg_kidx).  In the box every
// lane of a warp reads the same element-kernel word (a broadcast); in the
// spherical segment the lanes' elements lie in neighbouring (theta, r)
// columns, and the word-major table (kernels.h, GeoDF) puts their words next
// to each other.  The Gauss-point viscosities are pre-split into (hi, lo)
// pairs once per assembly.
#include <cuda_runtime.h>

#include <cstddef>

#include "kernels.h"

namespace {

#include "device.cuh"

// (sh, sl) += p + pl, p the leading part (Knuth's two-sum for sh + p)
__device__ __forceinline__ void df_add(float &sh, float &sl, float p, float pl)
{
	const float t = __fadd_rn(sh, p);
	const float bp = __fsub_rn(t, sh);
	const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
	sh = t;
	sl = __fadd_rn(sl, __fadd_rn(err, pl));
}

// (sh, sl) += (ah + al) (bh + bl), dropping al bl
__device__ __forceinline__ void df_madd(float &sh, float &sl, float ah, float al, float bh, float bl)
{
	const float p = __fmul_rn(ah, bh);
	const float e = __fmaf_rn(ah, bh, -p);  // the product's rounding error, exactly
	df_add(sh, sl, p, __fmaf_rn(ah, bl, __fmaf_rn(al, bh, e)));
}

__global__ void k_eta_split(int n, const double *__restrict__ evi, float2 *__restrict__ out)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
	{
		const double v = evi[i];
		const float h = (float)v;
		out[i] = make_float2(h, (float)(v - (double)h));
	}
}

constexpr int AS_THREADS = 256;
// the word offsets the kernel uses: mh, ml, lgh, lgl of GeoDF
static_assert(GEODF_WORDS == 2 * 4608 + 2 * 576, "GeoDF layout");
static_assert(offsetof(GeoDF, ml) == 4608 * sizeof(float) && offsetof(GeoDF, lgh) == 9216 * sizeof(float) &&
                  offsetof(GeoDF, lgl) == 9792 * sizeof(float),
              "GeoDF layout");

// YLANE (the spherical segment): the lanes of a warp are 32 nodes of one
// (x, z) line with the same y parity, so that all of them read the same
// column's element kernels (a broadcast, as in the box), at the price of
// stencil writes spread over 32 tiles.  Otherwise (the box) the lanes are the
// 32 positions of one stencil tile.
template <bool YLANE>
__global__ void __launch_bounds__(AS_THREADS) k_assemble_df(Lvl L, const float *__restrict__ G,
                                                           const float2 *__restrict__ eta2, int aug,
                                                           double *__restrict__ K64, float *__restrict__ K32,
                                                           float *__restrict__ K32lo, double *__restrict__ BI64,
                                                           float *__restrict__ BI32)
{
	pdl_begin();
	const int lane = threadIdx.x & 31;
	const long w = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int s = (int)(w % 27);
	int p, x, y, z;
	if constexpr(YLANE)
	{
		// warp (line, y parity, chunk of 32 y values of that parity, slot)
		const int nch = (L.cnt[1][0] + 31) / 32;
		long r = w / 27;
		const int chunk = (int)(r % nch);
		r /= nch;
		const int py = (int)(r % 2);
		r /= 2;
		if(r >= (long)L.nox * L.noz)
			return;
		z = (int)(r % L.noz);
		x = (int)(r / L.noz);
		y = py + 2 * (32 * chunk + lane);
		if(y >= L.noy)
			return;
		p = cg_pos(L, x, y, z);
	}
	else
	{
		const int tile = (int)(w / 27);
		if(tile >= L.toff[8])
			return;
		int c = 0;
#pragma unroll
		for(int k = 1; k < 8; ++k)
			c += (tile >= L.toff[k]);
		const int q = (tile - L.toff[c]) * CG_TILE + lane;
		if(q >= L.coff[c + 1] - L.coff[c])
			return;
		p = L.coff[c] + q;
		cg_decode(L, c, q, x, y, z);
	}
	const int dz = s % 3 - 1, dx = (s / 3) % 3 - 1, dy = s / 9 - 1;
	float bh[9], bl[9];
#pragma unroll
	for(int r = 0; r < 9; ++r)
		bh[r] = bl[r] = 0.f;
	const int mx = x + dx, my = y + dy, mz = z + dz;
	const bool inside = mx >= 0 && mx < L.nox && my >= 0 && my < L.noy && mz >= 0 && mz < L.noz;
	if(inside)
	{
		// elements holding both n and m: corner (ox, oy, oz) of n with (o + d) in {0, 1}
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
					const int a = cg_local_index(ox, oy, oz);
					const int b = cg_local_index(ox + dx, oy + dy, oz + dz);
					const float4 *ep = reinterpret_cast<const float4 *>(eta2 + 8 * (size_t)e);
					float eh[8], el[8];
#pragma unroll
					for(int k = 0; k < 4; ++k)
					{
						const float4 v = ep[k];
						eh[2 * k] = v.x;
						el[2 * k] = v.y;
						eh[2 * k + 1] = v.z;
						el[2 * k + 1] = v.w;
					}
					// word w of this element's column: Gc[w * ncol].  The box has
					// one column: constant strides and a warp-uniform address, so
					// its loads stay broadcasts
					const int ncol = YLANE ? L.elx * L.elz : 1;  // geo_count(L)
					const float *Gc = YLANE ? G + cg_col(L, x - ox, z - oz) : G;
#pragma unroll
					for(int k = 0; k < 8; ++k)
					{
						const size_t w0 = (size_t)(((k * 8 + a) * 8 + b) * 9);
#pragma unroll
						for(int r = 0; r < 9; ++r)
							df_madd(bh[r], bl[r], eh[k], el[k], Gc[(w0 + r) * ncol],
							        Gc[(4608 + w0 + r) * ncol]);
					}
					if(aug)
					{
						// mean viscosity (a pair), times lambda g_a,i g_b,j (pairs)
						float sh = 0.f, sl = 0.f;
#pragma unroll
						for(int k = 0; k < 8; ++k)
							df_add(sh, sl, eh[k], el[k]);
						sh *= 0.125f;
						sl *= 0.125f;
						const size_t g0 = (size_t)(9216 + (a * 8 + b) * 9);
#pragma unroll
						for(int r = 0; r < 9; ++r)
							df_madd(bh[r], bl[r], sh, sl, Gc[(g0 + r) * ncol], Gc[(576 + g0 + r) * ncol]);
					}
				}
			}
		}
	}
	if(s == 13)
	{
		// 1 / diag K from the unmasked diagonal
#pragma unroll
		for(int i = 0; i < 3; ++i)
		{
			const double bi = 1.0 / ((double)bh[4 * i] + (double)bl[4 * i]);
			if(BI64)
				BI64[3 * (size_t)p + i] = bi;
			if(BI32)
				BI32[3 * (size_t)p + i] = (float)bi;
		}
	}
	if(inside)
	{
		const unsigned fn = cg_vflag(L, x, y, z), fm = cg_vflag(L, mx, my, mz);
#pragma unroll
		for(int i = 0; i < 3; ++i)
#pragma unroll
			for(int j = 0; j < 3; ++j)
				if(((fn >> i) & 1u) || ((fm >> j) & 1u))
					bh[3 * i + j] = bl[3 * i + j] = 0.f;
	}
#pragma unroll
	for(int i = 0; i < 3; ++i)
#pragma unroll
		for(int j = 0; j < 3; ++j)
		{
			const int r = 3 * i + j;
			const size_t off = cg_kidx(L, s, i, j, p);
			// renormalised pair, in FP32 (two-sum): hi the entry rounded to
			// FP32, lo the exact remainder
			const float hi = __fadd_rn(bh[r], bl[r]);
			const float bp = __fsub_rn(hi, bh[r]);
			const float lo = __fadd_rn(__fsub_rn(bh[r], __fsub_rn(hi, bp)), __fsub_rn(bl[r], bp));
			if(K64)
				K64[off] = (double)bh[r] + (double)bl[r];
			if(K32)
				K32[off] = hi;
			if(K32lo)
				K32lo[off] = lo;
		}
}

template <typename... KArgs, typename... Args>
void as_launch(void (*kern)(KArgs...), int blocks, int threads, cudaStream_t st, Args... args)
{
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(blocks);
	cfg.blockDim = dim3(threads);
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = g_use_pdl ? 1 : 0;
	cudaLaunchKernelEx(&cfg, kern, ((KArgs)args)...);
	++g_kernel_launches;
}

} // namespace

void geo_df_fill(const Geo &g, int aug, double lambda, GeoDF *out)
{
	auto split = [](double v, float &h, float &l) {
		h = (float)v;
		l = (float)(v - (double)h);
	};
	for(int k = 0; k < 8; ++k)
		for(int a = 0; a < 8; ++a)
			for(int b = 0; b < 8; ++b)
				for(int r = 0; r < 9; ++r)
					split(g.Mk[k][a][b][r], out->mh[k][a][b][r], out->ml[k][a][b][r]);
	for(int a = 0; a < 8; ++a)
		for(int b = 0; b < 8; ++b)
			for(int r = 0; r < 9; ++r)
				split(aug ? lambda * g.g[3 * a + r / 3] * g.g[3 * b + r % 3] : 0.0, out->lgh[a][b][r], out->lgl[a][b][r]);
}

void launch_assemble_df(cudaStream_t st, const Lvl &L, const float *G, const double *evi, float2 *eta2, int aug,
                        double *K64, float *K32, float *K32lo, double *BI64, float *BI32)
{
	const int n = 8 * L.nel;
	as_launch(k_eta_split, (n + 255) / 256, 256, st, n, evi, eta2);
	if(L.sphere)  // one geometry column per (theta, r) element column: lanes along y
	{
		const long warps = 27L * 2 * ((L.cnt[1][0] + 31) / 32) * L.nox * L.noz;
		as_launch(k_assemble_df<true>, (int)((warps * 32 + AS_THREADS - 1) / AS_THREADS), AS_THREADS, st, L, G,
		          (const float2 *)eta2, aug, K64, K32, K32lo, BI64, BI32);
		return;
	}
	const long warps = 27L * L.toff[8];
	as_launch(k_assemble_df<false>, (int)((warps * 32 + AS_THREADS - 1) / AS_THREADS), AS_THREADS, st, L, G,
	          (const float2 *)eta2, aug, K64, K32, K32lo, BI64, BI32);
}
