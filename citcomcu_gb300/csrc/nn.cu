// Warm-start network of the Stokes solve: tensor-core convolution kernels
// (forward, backward-data, backward-weights), the grid transfers between its
// three resolutions, loss, Adam, and the kernels that move data between the
// solver's multigrid levels and the network grid.
//
// Convolutions are implicit GEMMs on the 5th-generation tensor cores.  A CTA
// of four warps owns 128 output rows (voxels for the forward and
// backward-data products, (tap, input channel) pairs for the weight
// gradient); per step its threads gather one operand tile pair into shared
// memory in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes per
// core matrix), one thread issues tcgen05.mma (BF16 x BF16 -> FP32, M = 128,
// N = output channels, K = 16 per instruction) into a tensor-memory
// accumulator and commits to an mbarrier, and the next tile pair is gathered
// into the other of two stages while the tensor core works.  The epilogue
// reads the accumulator with tcgen05.ld.  Every mbarrier wait is bounded: a
// wait that gives up sets an error word, the CTA waits (bounded) for the
// products it issued, frees its tensor memory and leaves.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "nn.h"

typedef __nv_bfloat16 bf16;

namespace {

#include "device.cuh"

// ------------------------------------------------------------------ layers
// resolution (0: the level's grid, 1: every other node, 2: every fourth),
// input and output channels, ReLU
struct LayerDef
{
	int res, cin, cout, relu;
};
constexpr LayerDef LD[NN_LAYERS] = {{0, 2, 16, 1},  {0, 16, 16, 1}, {1, 16, 32, 1}, {1, 32, 32, 1}, {2, 32, 64, 1},
                                    {2, 64, 64, 1}, {1, 64, 32, 1}, {0, 32, 16, 1}, {0, 16, 4, 0}};
inline int padc(int c) { return c < 16 ? 16 : c; }

__device__ int g_nn_err;  // 1 when a bounded wait of a tensor-core kernel gave up

// ------------------------------------------------------------------ tcgen05
__device__ __forceinline__ unsigned su32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, no swizzle: start address, leading byte
// offset (between core matrices adjacent along K), stride byte offset
// (between core matrices adjacent along M or N), descriptor version 1
__device__ __forceinline__ uint64_t sdesc(unsigned addr, unsigned lbo, unsigned sbo)
{
	return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N, M = 128
__device__ __forceinline__ unsigned idesc_bf16(int n) { return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) | (8u << 24); }

__device__ __forceinline__ void tc_alloc(unsigned dst, unsigned cols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(cols) : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(unsigned taddr, unsigned cols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_mma(unsigned d, uint64_t a, uint64_t b, unsigned idesc, unsigned acc)
{
	asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	             "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
	             "l"(a), "l"(b), "r"(idesc), "r"(acc)
	             : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void bar_init(unsigned bar) { asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory"); }

// bounded wait (at most about a second) for the phase of `bar` with this parity
__device__ __forceinline__ bool bar_wait(unsigned bar, unsigned parity)
{
	for(int it = 0; it < (1 << 20); ++it)
	{
		unsigned ok;
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(ok)
		             : "r"(bar), "r"(parity), "r"(1000u)
		             : "memory");
		if(ok)
			return true;
	}
	return false;
}

// 16 FP32 columns of the calling thread's tensor-memory lane
__device__ __forceinline__ void tc_ld16(unsigned taddr, float *v)
{
	unsigned r[16];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
	               "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	             : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for(int j = 0; j < 16; ++j)
		v[j] = __uint_as_float(r[j]);
}

// core matrix (row group g, K group k) of an operand with G row groups per
// K group: byte offset of the 16-byte row `r % 8`
__device__ __forceinline__ unsigned core_off(int kg, int rg, int G, int r8) { return (unsigned)((kg * G + rg) * 128 + r8 * 16); }

// ------------------------------------------------------------- convolution
struct ConvArgs
{
	const bf16 *x;      // [V][CIN]
	const bf16 *w;      // [27][COUT][CIN]
	const float *bias;  // [COUT] or null
	const bf16 *add;    // [V][COUT] or null: added before the activation
	const bf16 *mask;   // [V][COUT] or null: output zero where mask <= 0
	bf16 *y16;          // [V][COUT] (or null)
	float *y32;         // [V][COUT] (or null)
	int nx, ny, nz, V;
	int relu;
};

template <int CIN, int COUT> struct ConvCfg
{
	static constexpr int A = 128 * CIN * 2;
	static constexpr int B = COUT * CIN * 2;
	static constexpr int STAGE = A + B;
	static constexpr int COLS = COUT < 32 ? 32 : COUT;
	// + alignment slack; 64-column accumulators ask for at least 30 KB so that
	// no more than 7 CTAs (448 of the SM's 512 tensor-memory columns) share an SM
	static constexpr int SMEM = (2 * STAGE + 128) > (COLS == 64 ? 30 * 1024 : 0) ? (2 * STAGE + 128) : 30 * 1024;
};

// 3x3x3 convolution with zero padding: y[v][o] = sum_k sum_i x[v + off_k][i] w[k][o][i]
// (tap k = 9 (dy + 1) + 3 (dx + 1) + (dz + 1)), then + bias, + add, ReLU, mask.
template <int CIN, int COUT> __global__ void __launch_bounds__(128) k_nn_conv(const ConvArgs a)
{
	pdl_begin();
	using C = ConvCfg<CIN, COUT>;
	constexpr int KG = CIN / 8, NG = COUT / 8;
	extern __shared__ unsigned char smem_raw[];
	__shared__ __align__(8) unsigned long long bar[2];
	__shared__ unsigned tbase;
	unsigned char *sm = smem_raw + ((128 - (su32(smem_raw) & 127)) & 127);
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int v0 = blockIdx.x * 128;
	if(warp == 0)
		tc_alloc(su32(&tbase), C::COLS);
	if(tid == 0)
	{
		bar_init(su32(&bar[0]));
		bar_init(su32(&bar[1]));
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	tc_before();
	__syncthreads();
	tc_after();
	const unsigned tmem = tbase;
	int issued = 0;  // taps whose products were committed
	bool ok = true;
	for(int k = 0; k < 27; ++k)
	{
		const int b = k & 1;
		if(k >= 2)
		{
			// stage b is free once the products of tap k - 2 are done
			const bool w = bar_wait(su32(&bar[b]), (unsigned)(((k - 2) >> 1) & 1));
			if(!__syncthreads_and(w))
			{
				ok = false;
				break;
			}
		}
		unsigned char *sA = sm + b * C::STAGE, *sB = sA + C::A;
		const int dy = k / 9 - 1, dx = (k / 3) % 3 - 1, dz = k % 3 - 1;
		for(int c = tid; c < 128 * KG; c += 128)
		{
			const int m = c / KG, kg = c % KG, v = v0 + m;
			uint4 val = make_uint4(0u, 0u, 0u, 0u);
			if(v < a.V)
			{
				const int z = v % a.nz, t = v / a.nz, x = t % a.nx, y = t / a.nx;
				const int zz = z + dz, xx = x + dx, yy = y + dy;
				if(zz >= 0 && zz < a.nz && xx >= 0 && xx < a.nx && yy >= 0 && yy < a.ny)
					val = *reinterpret_cast<const uint4 *>(a.x + (size_t)(zz + a.nz * (xx + a.nx * yy)) * CIN + kg * 8);
			}
			*reinterpret_cast<uint4 *>(sA + core_off(kg, m >> 3, 16, m & 7)) = val;
		}
		const bf16 *wk = a.w + (size_t)k * COUT * CIN;
		for(int c = tid; c < COUT * KG; c += 128)
		{
			const int n = c / KG, kg = c % KG;
			*reinterpret_cast<uint4 *>(sB + core_off(kg, n >> 3, NG, n & 7)) = *reinterpret_cast<const uint4 *>(wk + (size_t)n * CIN + kg * 8);
		}
		// the generic-proxy stores above are read by the tensor core (async proxy)
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		__syncthreads();
		if(tid == 0)
		{
			tc_after();
#pragma unroll
			for(int kc = 0; kc < CIN / 16; ++kc)
				tc_mma(tmem, sdesc(su32(sA) + kc * 2 * 16 * 128, 16 * 128, 128), sdesc(su32(sB) + kc * 2 * NG * 128, NG * 128, 128),
				       idesc_bf16(COUT), (unsigned)(k | kc));
			tc_commit(su32(&bar[b]));
		}
		issued = k + 1;
	}
	// the last commit covers every product issued before it
	bool done = issued > 0 && bar_wait(su32(&bar[(issued - 1) & 1]), (unsigned)(((issued - 1) >> 1) & 1));
	done = __syncthreads_and(done) && ok;
	if(!done && tid == 0)
		atomicExch(&g_nn_err, 1);
	tc_after();
	if(done)
	{
		const int v = v0 + warp * 32 + lane;
#pragma unroll
		for(int c0 = 0; c0 < COUT; c0 += 16)
		{
			float acc[16];
			tc_ld16(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0, acc);
			if(v < a.V)
			{
				const size_t o = (size_t)v * COUT + c0;
				float out[16];
#pragma unroll
				for(int j = 0; j < 16; ++j)
				{
					float q = acc[j];
					if(a.bias)
						q += a.bias[c0 + j];
					if(a.add)
						q += __bfloat162float(a.add[o + j]);
					if(a.relu)
						q = fmaxf(q, 0.f);
					if(a.mask && !(__bfloat162float(a.mask[o + j]) > 0.f))
						q = 0.f;
					out[j] = q;
				}
				if(a.y32)
				{
#pragma unroll
					for(int j = 0; j < 16; j += 4)
						*reinterpret_cast<float4 *>(a.y32 + o + j) = make_float4(out[j], out[j + 1], out[j + 2], out[j + 3]);
				}
				else
				{
					__align__(16) bf16 hb[16];
#pragma unroll
					for(int j = 0; j < 16; ++j)
						hb[j] = __float2bfloat16_rn(out[j]);
					*reinterpret_cast<uint4 *>(a.y16 + o) = *reinterpret_cast<const uint4 *>(hb);
					*reinterpret_cast<uint4 *>(a.y16 + o + 8) = *reinterpret_cast<const uint4 *>(hb + 8);
				}
			}
		}
	}
	tc_before();
	__syncthreads();
	if(warp == 0)
		tc_dealloc(tmem, C::COLS);
}

// ------------------------------------------------------------ weight gradient
template <int CIN, int COUT> struct WgCfg
{
	static constexpr int TPT = 128 / CIN;           // taps per 128-row tile
	static constexpr int VS = 64;                   // voxels per stage (4 products of K = 16)
	static constexpr int A = 128 * VS * 2;
	static constexpr int B = COUT * VS * 2;
	static constexpr int STAGE = A + B;
	static constexpr int COLS = COUT < 32 ? 32 : COUT;
	static constexpr int SMEM = (2 * STAGE + 128) > (COLS == 64 ? 30 * 1024 : 0) ? (2 * STAGE + 128) : 30 * 1024;
};

// gw[k][o][i] += sum over the CTA's voxels v of x[v + off_k][i] dy[v][o]:
// rows (tap, input channel) of tile blockIdx.x, voxels of chunk blockIdx.y
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_nn_wgrad(const bf16 *x, const bf16 *dy, float *gw, int nx, int ny, int nz, int V, int vchunk)
{
	pdl_begin();
	using C = WgCfg<CIN, COUT>;
	constexpr int KG8 = CIN / 8, NG = COUT / 8, VS = C::VS;
	extern __shared__ unsigned char smem_raw[];
	__shared__ __align__(8) unsigned long long bar[2];
	__shared__ unsigned tbase;
	unsigned char *sm = smem_raw + ((128 - (su32(smem_raw) & 127)) & 127);
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int tile = blockIdx.x;
	const int vbeg = blockIdx.y * vchunk, vend = min(V, vbeg + vchunk);
	const int nst = vend > vbeg ? (vend - vbeg + VS - 1) / VS : 0;
	if(warp == 0)
		tc_alloc(su32(&tbase), C::COLS);
	if(tid == 0)
	{
		bar_init(su32(&bar[0]));
		bar_init(su32(&bar[1]));
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	tc_before();
	__syncthreads();
	tc_after();
	const unsigned tmem = tbase;
	int issued = 0;
	bool ok = true;
	for(int s = 0; s < nst; ++s)
	{
		const int b = s & 1;
		if(s >= 2)
		{
			const bool w = bar_wait(su32(&bar[b]), (unsigned)(((s - 2) >> 1) & 1));
			if(!__syncthreads_and(w))
			{
				ok = false;
				break;
			}
		}
		unsigned char *sA = sm + b * C::STAGE, *sB = sA + C::A;
		const int vs = vbeg + s * VS;
		// A: row r = t CIN + i (tap t of the tile, channel i), column = voxel
		for(int it = tid; it < VS * C::TPT * KG8; it += 128)
		{
			const int jj = it % VS, rest = it / VS, c8 = rest % KG8, t = rest / KG8;
			const int v = vs + jj, k = tile * C::TPT + t;
			uint4 val = make_uint4(0u, 0u, 0u, 0u);
			if(v < vend && k < 27)
			{
				const int z = v % nz, q = v / nz, xx0 = q % nx, yy0 = q / nx;
				const int zz = z + k % 3 - 1, xx = xx0 + (k / 3) % 3 - 1, yy = yy0 + k / 9 - 1;
				if(zz >= 0 && zz < nz && xx >= 0 && xx < nx && yy >= 0 && yy < ny)
					val = *reinterpret_cast<const uint4 *>(x + (size_t)(zz + nz * (xx + nx * yy)) * CIN + c8 * 8);
			}
			const bf16 *h = reinterpret_cast<const bf16 *>(&val);
			unsigned char *base = sA + core_off(jj >> 3, (t * CIN + 8 * c8) >> 3, 16, 0) + (jj & 7) * 2;
#pragma unroll
			for(int i = 0; i < 8; ++i)
				*reinterpret_cast<bf16 *>(base + i * 16) = h[i];
		}
		// B: row o (output channel), column = voxel
		for(int it = tid; it < VS * NG; it += 128)
		{
			const int jj = it % VS, c8 = it / VS, v = vs + jj;
			uint4 val = make_uint4(0u, 0u, 0u, 0u);
			if(v < vend)
				val = *reinterpret_cast<const uint4 *>(dy + (size_t)v * COUT + c8 * 8);
			const bf16 *h = reinterpret_cast<const bf16 *>(&val);
			unsigned char *base = sB + core_off(jj >> 3, c8, NG, 0) + (jj & 7) * 2;
#pragma unroll
			for(int i = 0; i < 8; ++i)
				*reinterpret_cast<bf16 *>(base + i * 16) = h[i];
		}
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		__syncthreads();
		if(tid == 0)
		{
			tc_after();
#pragma unroll
			for(int j = 0; j < VS / 16; ++j)
				tc_mma(tmem, sdesc(su32(sA) + j * 2 * 16 * 128, 16 * 128, 128), sdesc(su32(sB) + j * 2 * NG * 128, NG * 128, 128),
				       idesc_bf16(COUT), (unsigned)(s | j));
			tc_commit(su32(&bar[b]));
		}
		issued = s + 1;
	}
	bool done = issued > 0 && bar_wait(su32(&bar[(issued - 1) & 1]), (unsigned)(((issued - 1) >> 1) & 1));
	done = __syncthreads_and(done) && ok;
	if(!done && issued > 0 && tid == 0)
		atomicExch(&g_nn_err, 1);
	tc_after();
	if(done)
	{
		const int r = warp * 32 + lane, t = r / CIN, i = r % CIN, k = tile * C::TPT + t;
#pragma unroll
		for(int c0 = 0; c0 < COUT; c0 += 16)
		{
			float acc[16];
			tc_ld16(tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0, acc);
			if(k < 27)
#pragma unroll
				for(int j = 0; j < 16; ++j)
					atomicAdd(gw + ((size_t)k * COUT + c0 + j) * CIN + i, acc[j]);
		}
	}
	tc_before();
	__syncthreads();
	if(warp == 0)
		tc_dealloc(tmem, C::COLS);
}

// ------------------------------------------------------------ grid transfers
// 1D weight sum of coarse index i on nc nodes: 1 + 1/2 per existing neighbour
__device__ __forceinline__ float nrm1(int i, int nc) { return 1.f + 0.5f * (i > 0) + 0.5f * (i < nc - 1); }

// fine (2 nc - 1 per axis) <- coarse: trilinear prolongation, optionally of
// in / norm (the transpose of the normalised restriction), + add, mask
__global__ void k_nn_up(const bf16 *in, bf16 *out, const bf16 *add, const bf16 *mask, int cx, int cy, int cz, int C, int scale)
{
	pdl_begin();
	const int fx = 2 * cx - 1, fy = 2 * cy - 1, fz = 2 * cz - 1;
	const long n = (long)fx * fy * fz * C;
	for(long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
	{
		const int c = (int)(q % C);
		const int j = (int)(q / C);
		const int z = j % fz, t = j / fz, x = t % fx, y = t / fx;
		const int x0 = x >> 1, x1 = (x + 1) >> 1, y0 = y >> 1, y1 = (y + 1) >> 1, z0 = z >> 1, z1 = (z + 1) >> 1;
		float s = 0.f;
		for(int yy = y0; yy <= y1; ++yy)
			for(int xx = x0; xx <= x1; ++xx)
				for(int zz = z0; zz <= z1; ++zz)
				{
					const float w = ((x & 1) ? 0.5f : 1.f) * ((y & 1) ? 0.5f : 1.f) * ((z & 1) ? 0.5f : 1.f);
					float v = __bfloat162float(in[(size_t)(zz + cz * (xx + cx * yy)) * C + c]);
					if(scale)
						v /= nrm1(xx, cx) * nrm1(yy, cy) * nrm1(zz, cz);
					s += w * v;
				}
		if(add)
			s += __bfloat162float(add[q]);
		if(mask && !(__bfloat162float(mask[q]) > 0.f))
			s = 0.f;
		out[q] = __float2bfloat16_rn(s);
	}
}

// coarse <- fine: the transpose of the prolongation, optionally / norm (the
// normalised full-weighting restriction), + add, mask
__global__ void k_nn_down(const bf16 *in, bf16 *out, const bf16 *add, const bf16 *mask, int cx, int cy, int cz, int C, int scale)
{
	pdl_begin();
	const int fx = 2 * cx - 1, fy = 2 * cy - 1, fz = 2 * cz - 1;
	const long n = (long)cx * cy * cz * C;
	for(long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
	{
		const int c = (int)(q % C);
		const int I = (int)(q / C);
		const int z = I % cz, t = I / cz, x = t % cx, y = t / cx;
		float s = 0.f;
		for(int yy = max(2 * y - 1, 0); yy <= min(2 * y + 1, fy - 1); ++yy)
			for(int xx = max(2 * x - 1, 0); xx <= min(2 * x + 1, fx - 1); ++xx)
				for(int zz = max(2 * z - 1, 0); zz <= min(2 * z + 1, fz - 1); ++zz)
				{
					const float w = ((xx & 1) ? 0.5f : 1.f) * ((yy & 1) ? 0.5f : 1.f) * ((zz & 1) ? 0.5f : 1.f);
					s += w * __bfloat162float(in[(size_t)(zz + fz * (xx + fx * yy)) * C + c]);
				}
		if(scale)
			s /= nrm1(x, cx) * nrm1(y, cy) * nrm1(z, cz);
		if(add)
			s += __bfloat162float(add[q]);
		if(mask && !(__bfloat162float(mask[q]) > 0.f))
			s = 0.f;
		out[q] = __float2bfloat16_rn(s);
	}
}

// ------------------------------------------------------------ loss, bias, Adam
// dy = 2 scale (y - t) for the four used outputs (0 for the padding), loss += scale sum (y - t)^2
__global__ void k_nn_loss(const float *y, const float *t, bf16 *dy, int V, float scale, double *loss)
{
	pdl_begin();
	__shared__ float red[32];
	const int v = blockIdx.x * blockDim.x + threadIdx.x;
	float s = 0.f;
	if(v < V)
	{
#pragma unroll
		for(int c = 0; c < NN_CH; ++c)
		{
			float g = 0.f;
			if(c < NN_OUT)
			{
				const float d = y[(size_t)v * NN_CH + c] - t[(size_t)v * NN_OUT + c];
				s += d * d;
				g = 2.f * scale * d;
			}
			dy[(size_t)v * NN_CH + c] = __float2bfloat16_rn(g);
		}
	}
	for(int o = 16; o > 0; o >>= 1)
		s += __shfl_xor_sync(0xffffffffu, s, o);
	if((threadIdx.x & 31) == 0)
		red[threadIdx.x >> 5] = s;
	__syncthreads();
	if(threadIdx.x == 0)
	{
		float b = 0.f;
		for(int w = 0; w < (int)(blockDim.x >> 5); ++w)
			b += red[w];
		atomicAdd(loss, (double)b * (double)scale);
	}
}

// gb[c] += sum over voxels of g[v][c]
__global__ void k_nn_bgrad(const bf16 *g, int V, int C, float *gb)
{
	pdl_begin();
	const int c = threadIdx.x % C, r = threadIdx.x / C, rows = blockDim.x / C;
	float s = 0.f;
	for(int v = blockIdx.x * rows + r; v < V; v += gridDim.x * rows)
		s += __bfloat162float(g[(size_t)v * C + c]);
	atomicAdd(gb + c, s);
}

__global__ void k_nn_adam(float *w, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= n)
		return;
	const float gi = g[i];
	const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
	m[i] = mi;
	v[i] = vi;
	w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// BF16 copy of the master weights and the flipped, transposed copy that the
// backward-data convolution uses: wf[k][i][o] = w[26 - k][o][i]
__global__ void k_nn_cast(const float *w, bf16 *w16, bf16 *wf, int cout, int cin)
{
	pdl_begin();
	const int n = 27 * cout * cin;
	const int q = blockIdx.x * blockDim.x + threadIdx.x;
	if(q >= n)
		return;
	const int i = q % cin, o = (q / cin) % cout, k = q / (cin * cout);
	const bf16 b = __float2bfloat16_rn(w[q]);
	w16[q] = b;
	wf[((size_t)(26 - k) * cin + i) * cout + o] = b;
}

// ------------------------------------------------------- solver-side data
// work (FP64): [0, V) T restricted to the network grid, [V, V + nz) its
// horizontal means, [V + nz] the sum of squares of the anomaly, [V + nz + 1]
// the sum of the fine element pressures
__device__ __forceinline__ double anomaly_rms(const double *work, int V, int nz)
{
	const double a = sqrt(work[V + nz] / V);
	return a > 0.0 ? a : 0.0;
}

// restricted T (hat-weighted mean of the fine nodes within r - 1 of the coarse
// node along each axis, weights (r - |d|) / r) and the viscosity input: log10
// of the mean Gauss-point viscosity of the coarse elements around the node
__global__ void k_nn_inputs(Lvl Lf, Lvl Lc, int r, const double *T, const double *evi, bf16 *x16, double *work)
{
	pdl_begin();
	const int I = blockIdx.x * blockDim.x + threadIdx.x;
	if(I >= Lc.nno)
		return;
	const int z = I % Lc.noz, t = I / Lc.noz, x = t % Lc.nox, y = t / Lc.nox;
	double tw = 0.0, ws = 0.0;
	for(int dy = -(r - 1); dy <= r - 1; ++dy)
	{
		const int fy = r * y + dy;
		if(fy < 0 || fy >= Lf.noy)
			continue;
		for(int dx = -(r - 1); dx <= r - 1; ++dx)
		{
			const int fx = r * x + dx;
			if(fx < 0 || fx >= Lf.nox)
				continue;
			for(int dz = -(r - 1); dz <= r - 1; ++dz)
			{
				const int fz = r * z + dz;
				if(fz < 0 || fz >= Lf.noz)
					continue;
				const double w = (double)(r - abs(dx)) * (r - abs(dy)) * (r - abs(dz));
				tw += w * T[cg_node(Lf, fx, fy, fz)];
				ws += w;
			}
		}
	}
	work[I] = tw / ws;
	double s = 0.0;
	int cnt = 0;
	for(int ey = max(y - 1, 0); ey <= min(y, Lc.ely - 1); ++ey)
		for(int ex = max(x - 1, 0); ex <= min(x, Lc.elx - 1); ++ex)
			for(int ez = max(z - 1, 0); ez <= min(z, Lc.elz - 1); ++ez)
			{
				const int e = ez + Lc.elz * (ex + Lc.elx * ey);
				for(int g = 0; g < 8; ++g)
					s += evi[(size_t)e * 8 + g];
				cnt += 8;
			}
	bf16 *o = x16 + (size_t)I * NN_CH;
	o[1] = __float2bfloat16_rn((float)((log10(s / cnt) + 1.5) / 1.5));
	for(int c = 2; c < NN_CH; ++c)
		o[c] = __float2bfloat16_rn(0.f);
}

__device__ double block_sum(double v)
{
	__shared__ double red[32];
	for(int o = 16; o > 0; o >>= 1)
		v += __shfl_xor_sync(0xffffffffu, v, o);
	if((threadIdx.x & 31) == 0)
		red[threadIdx.x >> 5] = v;
	__syncthreads();
	double s = 0.0;
	if(threadIdx.x == 0)
		for(int w = 0; w < (int)(blockDim.x >> 5); ++w)
			s += red[w];
	return s;  // valid in thread 0
}

// one block per z: the horizontal mean of the restricted T; block 0 also
// clears the two sums that follow
__global__ void k_nn_zmean(Lvl Lc, double *work)
{
	pdl_begin();
	const int z = blockIdx.x, V = Lc.nno;
	double s = 0.0;
	for(int q = threadIdx.x; q < Lc.nox * Lc.noy; q += blockDim.x)
		s += work[z + Lc.noz * q];
	s = block_sum(s);
	if(threadIdx.x == 0)
	{
		work[V + z] = s / (Lc.nox * Lc.noy);
		if(z == 0)
		{
			work[V + Lc.noz] = 0.0;
			work[V + Lc.noz + 1] = 0.0;
		}
	}
}

__global__ void k_nn_anomaly_ss(Lvl Lc, double *work)
{
	pdl_begin();
	const int V = Lc.nno;
	double s = 0.0;
	for(int I = blockIdx.x * blockDim.x + threadIdx.x; I < V; I += gridDim.x * blockDim.x)
	{
		const double a = work[I] - work[V + I % Lc.noz];
		s += a * a;
	}
	s = block_sum(s);
	if(threadIdx.x == 0)
		atomicAdd(work + V + Lc.noz, s);
}

// network input 0: the temperature anomaly (T minus its horizontal mean) over its RMS
__global__ void k_nn_anomaly(Lvl Lc, const double *work, bf16 *x16)
{
	pdl_begin();
	const int I = blockIdx.x * blockDim.x + threadIdx.x, V = Lc.nno;
	if(I >= V)
		return;
	const double a = anomaly_rms(work, V, Lc.noz);
	const double v = a > 0.0 ? (work[I] - work[V + I % Lc.noz]) / a : 0.0;
	x16[(size_t)I * NN_CH] = __float2bfloat16_rn((float)v);
}

__global__ void k_nn_psum(Lvl Lf, int Vc, int nzc, const double *P, double *work)
{
	pdl_begin();
	double s = 0.0;
	for(int e = blockIdx.x * blockDim.x + threadIdx.x; e < Lf.nel; e += gridDim.x * blockDim.x)
		s += P[e];
	s = block_sum(s);
	if(threadIdx.x == 0)
		atomicAdd(work + Vc + nzc + 1, s);
}

// targets: U sampled at the coarse nodes / (su a), the nodal mean of the fine
// element pressures around the node minus the mean pressure, / (sp a), with
// a the anomaly RMS of the same state
__global__ void k_nn_targets(Lvl Lf, Lvl Lc, int r, const double *U, const double *P, double su, double sp, const double *work,
                             float *t)
{
	pdl_begin();
	const int I = blockIdx.x * blockDim.x + threadIdx.x;
	if(I >= Lc.nno)
		return;
	const double a0 = anomaly_rms(work, Lc.nno, Lc.noz), a = a0 > 0.0 ? a0 : 1.0;
	const double pm = work[Lc.nno + Lc.noz + 1] / Lf.nel;
	const int z = I % Lc.noz, q = I / Lc.noz, x = q % Lc.nox, y = q / Lc.nox;
	const int fx = r * x, fy = r * y, fz = r * z, j = cg_node(Lf, fx, fy, fz);
	double p = 0.0;
	int cnt = 0;
	for(int ey = max(fy - 1, 0); ey <= min(fy, Lf.ely - 1); ++ey)
		for(int ex = max(fx - 1, 0); ex <= min(fx, Lf.elx - 1); ++ex)
			for(int ez = max(fz - 1, 0); ez <= min(fz, Lf.elz - 1); ++ez)
			{
				p += P[ez + Lf.elz * (ex + Lf.elx * ey)];
				++cnt;
			}
	p /= cnt;
	float *o = t + (size_t)I * NN_OUT;
	o[0] = (float)(U[3 * (size_t)j] / (su * a));
	o[1] = (float)(U[3 * (size_t)j + 1] / (su * a));
	o[2] = (float)(U[3 * (size_t)j + 2] / (su * a));
	o[3] = (float)((p - pm) / (sp * a));
}

__global__ void k_nn_guess_u(Lvl Lc, const float *y, double su, const double *work, double *Uc)
{
	pdl_begin();
	const int I = blockIdx.x * blockDim.x + threadIdx.x;
	if(I >= Lc.nno)
		return;
	const double s = su * anomaly_rms(work, Lc.nno, Lc.noz);
	for(int d = 0; d < 3; ++d)
		Uc[3 * (size_t)I + d] = (double)y[(size_t)I * NN_CH + d] * s;
}

__global__ void k_nn_guess_p(Lvl Lf, Lvl Lc, int r, const float *y, double sp, double mp, const double *work, double *P)
{
	pdl_begin();
	// the scale once per block; the interpolation of the FP32 network output
	// in FP32 (per-element FP64 divisions and products ran at GB300's FP64 rate)
	__shared__ double s_sc;
	if(threadIdx.x == 0)
		s_sc = sp * anomaly_rms(work, Lc.nno, Lc.noz);
	__syncthreads();
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if(e >= Lf.nel)
		return;
	const int ez = e % Lf.elz, q = e / Lf.elz, ex = q % Lf.elx, ey = q / Lf.elx;
	// element centre in coarse-node units
	const float ir = 1.0f / (float)r;
	const float cxp = (ex + 0.5f) * ir, cyp = (ey + 0.5f) * ir, czp = (ez + 0.5f) * ir;
	const int x0 = min((int)cxp, Lc.nox - 2), y0 = min((int)cyp, Lc.noy - 2), z0 = min((int)czp, Lc.noz - 2);
	const float fx = cxp - x0, fy = cyp - y0, fz = czp - z0;
	float s = 0.f;
	for(int b = 0; b < 8; ++b)
	{
		const int dx = b & 1, dy = (b >> 1) & 1, dz = b >> 2;
		const float w = (dx ? fx : 1.f - fx) * (dy ? fy : 1.f - fy) * (dz ? fz : 1.f - fz);
		s += w * y[(size_t)cg_node(Lc, x0 + dx, y0 + dy, z0 + dz) * NN_CH + 3];
	}
	P[e] = (double)s * s_sc + mp;
}

} // namespace

// ====================================================================== host

namespace {

int nblk(long n, int t = 256) { return (int)((n + t - 1) / t); }

template <typename... KArgs, typename... Args>
void launch_nn(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args)
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

// activations: input, encoder, bottleneck, decoder
enum Act
{
	X0, A1, A2, B0, B1, B2, C0, C1, C2, D0, D1, E0, E1, NACT
};
constexpr int ACT_RES[NACT] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 1, 1, 0, 0};
constexpr int ACT_C[NACT] = {16, 16, 16, 16, 32, 32, 32, 64, 64, 64, 32, 32, 16};
// gradients (of the pre-activation where a ReLU follows)
enum Grad
{
	GY, GE1, GE0, GD1, GD0, GC2, GC1, GC0, GB2, GB1, GB0, GA2, GA1, NGRAD
};
constexpr int GRAD_RES[NGRAD] = {0, 0, 0, 1, 1, 2, 2, 2, 1, 1, 1, 0, 0};
constexpr int GRAD_C[NGRAD] = {16, 16, 32, 32, 64, 64, 64, 32, 32, 32, 16, 16, 16};

bool g_attrs_done = false;

template <int CI, int CO> int conv_attr()
{
	int e = (int)cudaFuncSetAttribute(k_nn_conv<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, ConvCfg<CI, CO>::SMEM);
	e |= (int)cudaFuncSetAttribute(k_nn_wgrad<CI, CO>, cudaFuncAttributeMaxDynamicSharedMemorySize, WgCfg<CI, CO>::SMEM);
	return e;
}

int nn_attrs()
{
	if(g_attrs_done)
		return 0;
	int e = conv_attr<16, 16>() | conv_attr<16, 32>() | conv_attr<32, 16>() | conv_attr<32, 32>() | conv_attr<32, 64>() |
	        conv_attr<64, 32>() | conv_attr<64, 64>();
	if(e == 0)
		g_attrs_done = true;
	return e;
}

} // namespace

struct NnNet
{
	int nx[3], ny[3], nz[3], V[3];
	cudaStream_t st;
	size_t woff[NN_LAYERS], boff[NN_LAYERS], nflat;
	int cinP[NN_LAYERS], coutP[NN_LAYERS];
	float *master, *grad, *m1, *m2;
	bf16 *w16, *wf;
	bf16 *act[NACT];
	bf16 *g[NGRAD];
	float *y32;
	double *loss;
	int adam_t;
	std::vector<void *> allocs;
};

namespace {

template <typename T> int nalloc(NnNet *n, T **p, size_t count)
{
	void *q = nullptr;
	if(cudaMalloc(&q, (count ? count : 1) * sizeof(T)) != cudaSuccess)
		return -1;
	cudaMemset(q, 0, (count ? count : 1) * sizeof(T));
	n->allocs.push_back(q);
	*p = (T *)q;
	return 0;
}

void conv(NnNet *n, int cin, int cout, const ConvArgs &a)
{
	const dim3 grid((a.V + 127) / 128);
#define NN_CONV(CI, CO)                                                                                          \
	if(cin == CI && cout == CO)                                                                                  \
	{                                                                                                            \
		launch_nn(k_nn_conv<CI, CO>, grid, dim3(128), (size_t)ConvCfg<CI, CO>::SMEM, n->st, a);                  \
		return;                                                                                                  \
	}
	NN_CONV(16, 16)
	NN_CONV(16, 32)
	NN_CONV(32, 16)
	NN_CONV(32, 32)
	NN_CONV(32, 64)
	NN_CONV(64, 32)
	NN_CONV(64, 64)
#undef NN_CONV
}

void wgrad(NnNet *n, int cin, int cout, const bf16 *x, const bf16 *dy, float *gw, int res)
{
	const int V = n->V[res], vchunk = 2048;
	const dim3 grid((27 * cin + 127) / 128, (V + vchunk - 1) / vchunk);
#define NN_WG(CI, CO)                                                                                                          \
	if(cin == CI && cout == CO)                                                                                                \
	{                                                                                                                          \
		launch_nn(k_nn_wgrad<CI, CO>, grid, dim3(128), (size_t)WgCfg<CI, CO>::SMEM, n->st, x, dy, gw, n->nx[res], n->ny[res], \
		          n->nz[res], V, vchunk);                                                                                      \
		return;                                                                                                                \
	}
	NN_WG(16, 16)
	NN_WG(16, 32)
	NN_WG(32, 16)
	NN_WG(32, 32)
	NN_WG(32, 64)
	NN_WG(64, 32)
	NN_WG(64, 64)
#undef NN_WG
}

ConvArgs cargs(NnNet *n, int res, const bf16 *x, const bf16 *w)
{
	ConvArgs a;
	memset(&a, 0, sizeof(a));
	a.x = x;
	a.w = w;
	a.nx = n->nx[res];
	a.ny = n->ny[res];
	a.nz = n->nz[res];
	a.V = n->V[res];
	return a;
}

// forward convolution of layer l
void fwd(NnNet *n, int l, const bf16 *x, bf16 *y16, float *y32, const bf16 *add)
{
	ConvArgs a = cargs(n, LD[l].res, x, n->w16 + n->woff[l]);
	a.bias = n->master + n->boff[l];
	a.add = add;
	a.relu = LD[l].relu;
	a.y16 = y16;
	a.y32 = y32;
	conv(n, n->cinP[l], n->coutP[l], a);
}

// backward-data convolution of layer l: dx = conv(dy, flipped w) (+ add), mask
void bwd_data(NnNet *n, int l, const bf16 *dy, bf16 *dx, const bf16 *mask)
{
	ConvArgs a = cargs(n, LD[l].res, dy, n->wf + n->woff[l]);
	a.mask = mask;
	a.y16 = dx;
	conv(n, n->coutP[l], n->cinP[l], a);
}

void bwd_weights(NnNet *n, int l, const bf16 *x, const bf16 *dy)
{
	const int res = LD[l].res, C = n->coutP[l];
	wgrad(n, n->cinP[l], C, x, dy, n->grad + n->woff[l], res);
	const int rows = 256 / C;
	launch_nn(k_nn_bgrad, dim3(std::min(nblk(n->V[res], rows), 152)), dim3(256), 0, n->st, (const bf16 *)dy, n->V[res], C,
	          n->grad + n->boff[l]);
}

// res r (fine) <- res r + 1 (coarse)
void up(NnNet *n, int r, const bf16 *in, bf16 *out, int C, int scale, const bf16 *add, const bf16 *mask)
{
	launch_nn(k_nn_up, dim3(std::min(nblk((long)n->V[r] * C), 4096)), dim3(256), 0, n->st, in, out, add, mask, n->nx[r + 1],
	          n->ny[r + 1], n->nz[r + 1], C, scale);
}

// res r + 1 (coarse) <- res r (fine)
void down(NnNet *n, int r, const bf16 *in, bf16 *out, int C, int scale, const bf16 *add, const bf16 *mask)
{
	launch_nn(k_nn_down, dim3(std::min(nblk((long)n->V[r + 1] * C), 4096)), dim3(256), 0, n->st, in, out, add, mask, n->nx[r + 1],
	          n->ny[r + 1], n->nz[r + 1], C, scale);
}

void forward_into(NnNet *n, const bf16 *x0, float *y32)
{
	bf16 **a = n->act;
	fwd(n, 0, x0, a[A1], nullptr, nullptr);
	fwd(n, 1, a[A1], a[A2], nullptr, nullptr);
	down(n, 0, a[A2], a[B0], 16, 1, nullptr, nullptr);
	fwd(n, 2, a[B0], a[B1], nullptr, nullptr);
	fwd(n, 3, a[B1], a[B2], nullptr, nullptr);
	down(n, 1, a[B2], a[C0], 32, 1, nullptr, nullptr);
	fwd(n, 4, a[C0], a[C1], nullptr, nullptr);
	fwd(n, 5, a[C1], a[C2], nullptr, nullptr);
	up(n, 1, a[C2], a[D0], 64, 0, nullptr, nullptr);
	fwd(n, 6, a[D0], a[D1], nullptr, a[B2]);
	up(n, 0, a[D1], a[E0], 32, 0, nullptr, nullptr);
	fwd(n, 7, a[E0], a[E1], nullptr, a[A2]);
	fwd(n, 8, a[E1], nullptr, y32, nullptr);
}

void recast(NnNet *n)
{
	for(int l = 0; l < NN_LAYERS; ++l)
	{
		const int cnt = 27 * n->coutP[l] * n->cinP[l];
		launch_nn(k_nn_cast, dim3(nblk(cnt)), dim3(256), 0, n->st, (const float *)(n->master + n->woff[l]), n->w16 + n->woff[l],
		          n->wf + n->woff[l], n->coutP[l], n->cinP[l]);
	}
}

// deterministic uniform numbers in [-1, 1) (the same on every host)
struct Lcg
{
	uint64_t s;
	double next()
	{
		s = s * 6364136223846793005ull + 1442695040888963407ull;
		return ((double)(s >> 11) / 9007199254740992.0) * 2.0 - 1.0;
	}
};

} // namespace

int nn_create(int nx, int ny, int nz, unsigned seed, cudaStream_t st, NnNet **out, char *err, size_t errlen)
{
	*out = nullptr;
	if(nx < 9 || ny < 9 || nz < 9 || (nx - 1) % 4 || (ny - 1) % 4 || (nz - 1) % 4)
	{
		snprintf(err, errlen, "network grid %dx%dx%d: every axis needs (n - 1) divisible by 4 and n >= 9", nx, ny, nz);
		return -1;
	}
	if(nn_attrs() != 0)
	{
		snprintf(err, errlen, "network kernel attributes could not be set");
		return -1;
	}
	NnNet *n = new NnNet();
	n->st = st;
	n->nx[0] = nx;
	n->ny[0] = ny;
	n->nz[0] = nz;
	for(int r = 1; r < 3; ++r)
	{
		n->nx[r] = (n->nx[r - 1] - 1) / 2 + 1;
		n->ny[r] = (n->ny[r - 1] - 1) / 2 + 1;
		n->nz[r] = (n->nz[r - 1] - 1) / 2 + 1;
	}
	for(int r = 0; r < 3; ++r)
		n->V[r] = n->nx[r] * n->ny[r] * n->nz[r];
	size_t off = 0;
	for(int l = 0; l < NN_LAYERS; ++l)
	{
		n->cinP[l] = padc(LD[l].cin);
		n->coutP[l] = padc(LD[l].cout);
		n->woff[l] = off;
		off += (size_t)27 * n->cinP[l] * n->coutP[l];
		n->boff[l] = off;
		off += n->coutP[l];
		off = (off + 7) / 8 * 8;  // keeps every weight block 16-byte aligned in BF16
	}
	n->nflat = off;
	bool bad = nalloc(n, &n->master, off) || nalloc(n, &n->grad, off) || nalloc(n, &n->m1, off) || nalloc(n, &n->m2, off) ||
	           nalloc(n, &n->w16, off) || nalloc(n, &n->wf, off) || nalloc(n, &n->y32, (size_t)n->V[0] * NN_CH) ||
	           nalloc(n, &n->loss, 1);
	for(int i = 0; i < NACT && !bad; ++i)
		bad = nalloc(n, &n->act[i], (size_t)n->V[ACT_RES[i]] * ACT_C[i]) != 0;
	for(int i = 0; i < NGRAD && !bad; ++i)
		bad = nalloc(n, &n->g[i], (size_t)n->V[GRAD_RES[i]] * GRAD_C[i]) != 0;
	if(bad)
	{
		snprintf(err, errlen, "network buffers could not be allocated");
		nn_destroy(n);
		return -1;
	}
	// He-uniform initial weights over the used channels, zero biases; the
	// output layer starts small
	std::vector<float> h(off, 0.f);
	Lcg rng{0x9E3779B97F4A7C15ull ^ (uint64_t)seed};
	for(int l = 0; l < NN_LAYERS; ++l)
	{
		const double a = std::sqrt(6.0 / (27.0 * LD[l].cin)) * (l == NN_LAYERS - 1 ? 0.1 : 1.0);
		for(int o = 0; o < LD[l].cout; ++o)
			for(int i = 0; i < LD[l].cin; ++i)
				for(int k = 0; k < 27; ++k)
					h[n->woff[l] + ((size_t)k * n->coutP[l] + o) * n->cinP[l] + i] = (float)(a * rng.next());
	}
	cudaMemcpyAsync(n->master, h.data(), off * sizeof(float), cudaMemcpyHostToDevice, st);
	recast(n);
	if(cudaStreamSynchronize(st) != cudaSuccess)
	{
		snprintf(err, errlen, "network set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
		nn_destroy(n);
		return -1;
	}
	*out = n;
	return 0;
}

void nn_destroy(NnNet *n)
{
	if(!n)
		return;
	cudaStreamSynchronize(n->st);
	for(void *p : n->allocs)
		cudaFree(p);
	delete n;
}

int nn_param_count(const NnNet *n)
{
	int c = 0;
	(void)n;
	for(int l = 0; l < NN_LAYERS; ++l)
		c += 27 * LD[l].cin * LD[l].cout + LD[l].cout;
	return c;
}

int nn_voxels(const NnNet *n) { return n->V[0]; }

namespace {

// public layout (per layer W[o][i][27], b[o]) <-> padded flat layout
void pack(const NnNet *n, const float *flat, float *pub)
{
	size_t p = 0;
	for(int l = 0; l < NN_LAYERS; ++l)
	{
		for(int o = 0; o < LD[l].cout; ++o)
			for(int i = 0; i < LD[l].cin; ++i)
				for(int k = 0; k < 27; ++k)
					pub[p++] = flat[n->woff[l] + ((size_t)k * n->coutP[l] + o) * n->cinP[l] + i];
		for(int o = 0; o < LD[l].cout; ++o)
			pub[p++] = flat[n->boff[l] + o];
	}
}

void unpack(const NnNet *n, const float *pub, float *flat)
{
	size_t p = 0;
	for(int l = 0; l < NN_LAYERS; ++l)
	{
		for(int o = 0; o < LD[l].cout; ++o)
			for(int i = 0; i < LD[l].cin; ++i)
				for(int k = 0; k < 27; ++k)
					flat[n->woff[l] + ((size_t)k * n->coutP[l] + o) * n->cinP[l] + i] = pub[p++];
		for(int o = 0; o < LD[l].cout; ++o)
			flat[n->boff[l] + o] = pub[p++];
	}
}

int fetch_flat(NnNet *n, const float *dev, float *pub)
{
	std::vector<float> h(n->nflat);
	if(cudaMemcpyAsync(h.data(), dev, n->nflat * sizeof(float), cudaMemcpyDeviceToHost, n->st) != cudaSuccess ||
	   cudaStreamSynchronize(n->st) != cudaSuccess)
		return -1;
	pack(n, h.data(), pub);
	return 0;
}

} // namespace

int nn_get_params(NnNet *n, float *host) { return fetch_flat(n, n->master, host); }
int nn_get_grads(NnNet *n, float *host) { return fetch_flat(n, n->grad, host); }

int nn_set_params(NnNet *n, const float *host)
{
	std::vector<float> h(n->nflat, 0.f);
	unpack(n, host, h.data());
	if(cudaMemcpyAsync(n->master, h.data(), n->nflat * sizeof(float), cudaMemcpyHostToDevice, n->st) != cudaSuccess)
		return -1;
	recast(n);
	// fresh optimiser state for the new weights
	cudaMemsetAsync(n->m1, 0, n->nflat * sizeof(float), n->st);
	cudaMemsetAsync(n->m2, 0, n->nflat * sizeof(float), n->st);
	n->adam_t = 0;
	return cudaStreamSynchronize(n->st) == cudaSuccess ? 0 : -1;
}

int nn_forward(NnNet *n, const void *x16, float *y32)
{
	forward_into(n, (const bf16 *)x16, y32);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

const float *nn_last_output(const NnNet *n) { return n->y32; }

int nn_zero_grads(NnNet *n)
{
	cudaMemsetAsync(n->grad, 0, n->nflat * sizeof(float), n->st);
	cudaMemsetAsync(n->loss, 0, sizeof(double), n->st);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int nn_accumulate(NnNet *n, const void *x16, const float *t, float scale)
{
	const bf16 *x0 = (const bf16 *)x16;
	bf16 **a = n->act, **g = n->g;
	forward_into(n, x0, n->y32);
	launch_nn(k_nn_loss, dim3(nblk(n->V[0])), dim3(256), 0, n->st, (const float *)n->y32, t, g[GY], n->V[0], scale, n->loss);
	// head: y = conv(e1)
	bwd_weights(n, 8, a[E1], g[GY]);
	bwd_data(n, 8, g[GY], g[GE1], a[E1]);            // d(e1 pre-activation)
	// e1 = relu(conv(e0) + a2)
	bwd_weights(n, 7, a[E0], g[GE1]);
	bwd_data(n, 7, g[GE1], g[GE0], nullptr);
	down(n, 0, g[GE0], g[GD1], 32, 0, nullptr, a[D1]);  // through e0 = P(d1), then d1's ReLU
	// d1 = relu(conv(d0) + b2)
	bwd_weights(n, 6, a[D0], g[GD1]);
	bwd_data(n, 6, g[GD1], g[GD0], nullptr);
	down(n, 1, g[GD0], g[GC2], 64, 0, nullptr, a[C2]);  // through d0 = P(c2)
	bwd_weights(n, 5, a[C1], g[GC2]);
	bwd_data(n, 5, g[GC2], g[GC1], a[C1]);
	bwd_weights(n, 4, a[C0], g[GC1]);
	bwd_data(n, 4, g[GC1], g[GC0], nullptr);
	up(n, 1, g[GC0], g[GB2], 32, 1, g[GD1], a[B2]);      // through c0 = R(b2), plus the skip into d1
	bwd_weights(n, 3, a[B1], g[GB2]);
	bwd_data(n, 3, g[GB2], g[GB1], a[B1]);
	bwd_weights(n, 2, a[B0], g[GB1]);
	bwd_data(n, 2, g[GB1], g[GB0], nullptr);
	up(n, 0, g[GB0], g[GA2], 16, 1, g[GE1], a[A2]);      // through b0 = R(a2), plus the skip into e1
	bwd_weights(n, 1, a[A1], g[GA2]);
	bwd_data(n, 1, g[GA2], g[GA1], a[A1]);
	bwd_weights(n, 0, x0, g[GA1]);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int nn_adam(NnNet *n, float lr, float beta1, float beta2, float eps)
{
	n->adam_t += 1;
	const float c1 = 1.f - std::pow(beta1, (float)n->adam_t), c2 = 1.f - std::pow(beta2, (float)n->adam_t);
	launch_nn(k_nn_adam, dim3(nblk((long)n->nflat)), dim3(256), 0, n->st, n->master, (const float *)n->grad, n->m1, n->m2,
	          (int)n->nflat, lr, beta1, beta2, eps, c1, c2);
	recast(n);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int nn_loss(NnNet *n, double *loss)
{
	if(cudaMemcpyAsync(loss, n->loss, sizeof(double), cudaMemcpyDeviceToHost, n->st) != cudaSuccess ||
	   cudaStreamSynchronize(n->st) != cudaSuccess)
		return -1;
	return 0;
}

int nn_device_error(NnNet *n)
{
	int e = 0;
	cudaStreamSynchronize(n->st);
	if(cudaMemcpyFromSymbol(&e, g_nn_err, sizeof(int)) != cudaSuccess)
		return -1;
	return e;
}

void launch_nn_inputs(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, int r, const double *T, const double *evi_c, void *x16,
                      double *work)
{
	launch_nn(k_nn_inputs, dim3(nblk(Lc.nno)), dim3(256), 0, st, Lf, Lc, r, T, evi_c, (bf16 *)x16, work);
	launch_nn(k_nn_zmean, dim3(Lc.noz), dim3(256), 0, st, Lc, work);
	launch_nn(k_nn_anomaly_ss, dim3(std::min(nblk(Lc.nno), 64)), dim3(256), 0, st, Lc, work);
	launch_nn(k_nn_anomaly, dim3(nblk(Lc.nno)), dim3(256), 0, st, Lc, (const double *)work, (bf16 *)x16);
}

void launch_nn_targets(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, int r, const double *U, const double *P, double su,
                       double sp, double *work, float *t)
{
	launch_nn(k_nn_psum, dim3(std::min(nblk(Lf.nel), 64)), dim3(256), 0, st, Lf, Lc.nno, Lc.noz, P, work);
	launch_nn(k_nn_targets, dim3(nblk(Lc.nno)), dim3(256), 0, st, Lf, Lc, r, U, P, su, sp, (const double *)work, t);
}

void launch_nn_guess(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, int r, const float *y32, double su, double sp, double mp,
                     const double *work, double *Uc, double *P)
{
	launch_nn(k_nn_guess_u, dim3(nblk(Lc.nno)), dim3(256), 0, st, Lc, y32, su, work, Uc);
	launch_nn(k_nn_guess_p, dim3(nblk(Lf.nel)), dim3(256), 0, st, Lf, Lc, r, y32, sp, mp, work, P);
}
