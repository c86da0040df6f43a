// Matrix-free Gauss-Seidel colour of the FP32 multigrid on the box levels.
//
// The stored-stencil smoother (tile.cu) streams 243 coefficients per node and
// colour from HBM.  This kernel applies the operator from the viscosity at
// the Gauss points instead, as e_assemble_del2_u does element by element
// (Element_calculations.c:494-545): for the box the element matrix of
// get_elt_k (:133-293, Cartesian branch) is
//   K_ab[i][j] = sum_k J eta_k (dN_a/dx_j dN_b/dx_i + delta_ij grad N_a . grad N_b)
// (+ the augmented term lambda mean(eta) g_a,i g_b,j of get_aug_k, :1127-1163),
// so row (a, i) applied to the element's velocities d_b is
//   sum_k J eta_k sum_j dN_a/dx_j (G_ij + G_ji),  G_ij = d(d_i)/dx_j at point k.
// The gradient at the eight Gauss points is formed by sum factorisation: the
// x derivative of a trilinear field does not depend on x, so it is the
// difference of the two x faces interpolated bilinearly to the 2 x 2 (y, z)
// Gauss points (and likewise for y and z): 20 operations per component and
// direction instead of 64.
//
// Work split: eight threads per node of the colour, one per element around
// it.  No two nodes of a colour share an element, so the elements of a colour
// launch are disjoint; the eight row contributions of a node are added by
// three warp shuffles inside its group of eight lanes (no atomics), and the
// group's first lane updates the node.  Reads per node and colour: the
// 27-node neighbourhood of d (L1/L2-resident), F, 1/diag K, and the Gauss-point
// viscosity of its eight elements (32 B each, FP32).  Constrained dofs: rows
// are not updated, columns are masked on load (the reference zeroes both in
// construct_node_ks).
#include <cuda_runtime.h>

#include "kernels.h"

namespace {

#include "device.cuh"

constexpr int MF_THREADS = 256;
constexpr float GA = 0.78867513459481288225f;  // (1 + 1/sqrt 3) / 2: 1D shape function at its own Gauss point
constexpr float GB = 0.21132486540518711775f;  // (1 - 1/sqrt 3) / 2: at the other one

// corner values v[i0][i1] over two axes -> values at the 2 x 2 Gauss points
// of those axes (o[p0][p1]), phi_i(p) = GA if i == p else GB
__device__ __forceinline__ void mf_bilin(float v00, float v01, float v10, float v11, float o[2][2])
{
	const float a0 = GA * v00 + GB * v10, b0 = GB * v00 + GA * v10;  // axis 0 at p0 = 0, 1; axis 1 at i1 = 0
	const float a1 = GA * v01 + GB * v11, b1 = GB * v01 + GA * v11;  // i1 = 1
	o[0][0] = GA * a0 + GB * a1;
	o[0][1] = GB * a0 + GA * a1;
	o[1][0] = GA * b0 + GB * b1;
	o[1][1] = GB * b0 + GA * b1;
}

__device__ __forceinline__ float mf_phi(int i, int p) { return i == p ? GA : GB; }

template <bool AUG>
__global__ void __launch_bounds__(MF_THREADS) k_mf_gs(Lvl L, const float *__restrict__ eta, const float *__restrict__ BI,
                                                    const float *__restrict__ F, float *d, int colour, float lambda)
{
	pdl_begin();
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	const int q = t >> 3, a = t & 7;  // node of the colour; its local index in this thread's element
	const int ncol = L.coff[colour + 1] - L.coff[colour];
	const bool node_ok = q < ncol;
	int x = 0, y = 0, z = 0;
	if(node_ok)
		cg_decode(L, colour, q, x, y, z);
	const int ax = cg_loc(a, 0), ay = cg_loc(a, 1), az = cg_loc(a, 2);
	const int ex = x - ax, ey = y - ay, ez = z - az;
	const bool el_ok = node_ok && ex >= 0 && ex < L.elx && ey >= 0 && ey < L.ely && ez >= 0 && ez < L.elz;
	float y0 = 0.f, y1 = 0.f, y2 = 0.f;
	if(el_ok)
	{
		const float ih[3] = {(float)(1.0 / L.h[0]), (float)(1.0 / L.h[1]), (float)(1.0 / L.h[2])};
		const float J = (float)L.J;
		// the element's velocities u[ix][iy][iz][c], constrained dofs masked
		float u[2][2][2][3];
#pragma unroll
		for(int b = 0; b < 8; ++b)
		{
			const int bx = b & 1, by = (b >> 1) & 1, bz = b >> 2;
			const int nx = ex + bx, ny = ey + by, nz = ez + bz;
			const int n = cg_node(L, nx, ny, nz);
			const unsigned fl = cg_vflag(L, nx, ny, nz);
			u[bx][by][bz][0] = (fl & 1u) ? 0.f : d[3 * n];
			u[bx][by][bz][1] = (fl & 2u) ? 0.f : d[3 * n + 1];
			u[bx][by][bz][2] = (fl & 4u) ? 0.f : d[3 * n + 2];
		}
		const int e = ez + L.elz * (ex + L.elx * ey);
		const float4 e0 = reinterpret_cast<const float4 *>(eta)[2 * e], e1 = reinterpret_cast<const float4 *>(eta)[2 * e + 1];
		const float et[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
		// gradients at the Gauss points: gx[c][py][pz] = d u_c / dx (independent of px), etc.
		float gx[3][2][2], gy[3][2][2], gz[3][2][2];
#pragma unroll
		for(int c = 0; c < 3; ++c)
		{
			mf_bilin(ih[0] * (u[1][0][0][c] - u[0][0][0][c]), ih[0] * (u[1][0][1][c] - u[0][0][1][c]),
			         ih[0] * (u[1][1][0][c] - u[0][1][0][c]), ih[0] * (u[1][1][1][c] - u[0][1][1][c]), gx[c]);
			mf_bilin(ih[1] * (u[0][1][0][c] - u[0][0][0][c]), ih[1] * (u[0][1][1][c] - u[0][0][1][c]),
			         ih[1] * (u[1][1][0][c] - u[1][0][0][c]), ih[1] * (u[1][1][1][c] - u[1][0][1][c]), gy[c]);
			mf_bilin(ih[2] * (u[0][0][1][c] - u[0][0][0][c]), ih[2] * (u[0][1][1][c] - u[0][1][0][c]),
			         ih[2] * (u[1][0][1][c] - u[1][0][0][c]), ih[2] * (u[1][1][1][c] - u[1][1][0][c]), gz[c]);
		}
		float emean = 0.f;
#pragma unroll
		for(int k = 0; k < 8; ++k)
		{
			const int px = cg_loc(k, 0), py = cg_loc(k, 1), pz = cg_loc(k, 2);
			emean += et[k];
			// G[i][j] = d u_i / dx_j at this point
			const float G00 = gx[0][py][pz], G01 = gy[0][px][pz], G02 = gz[0][px][py];
			const float G10 = gx[1][py][pz], G11 = gy[1][px][pz], G12 = gz[1][px][py];
			const float G20 = gx[2][py][pz], G21 = gy[2][px][pz], G22 = gz[2][px][py];
			const float S01 = G01 + G10, S02 = G02 + G20, S12 = G12 + G21;
			// J eta_k grad N_a at this point
			const float w = J * et[k];
			const float fx = mf_phi(ax, px), fy = mf_phi(ay, py), fz = mf_phi(az, pz);
			const float n0 = w * (ax ? ih[0] : -ih[0]) * fy * fz;
			const float n1 = w * (ay ? ih[1] : -ih[1]) * fx * fz;
			const float n2 = w * (az ? ih[2] : -ih[2]) * fx * fy;
			y0 += n0 * (2.f * G00) + n1 * S01 + n2 * S02;
			y1 += n0 * S01 + n1 * (2.f * G11) + n2 * S12;
			y2 += n0 * S02 + n1 * S12 + n2 * (2.f * G22);
		}
		if(AUG)
		{
			// g_b,i = -8 J dN_b/dx_i at the centre = -2 J s_b,i / h_i (get_elt_g)
			float gd = 0.f;
#pragma unroll
			for(int c = 0; c < 3; ++c)
			{
				float s = 0.f;
#pragma unroll
				for(int b = 0; b < 8; ++b)
				{
					const int bb[3] = {b & 1, (b >> 1) & 1, b >> 2};
					s += bb[c] ? u[b & 1][(b >> 1) & 1][b >> 2][c] : -u[b & 1][(b >> 1) & 1][b >> 2][c];
				}
				gd += ih[c] * s;
			}
			gd *= -2.f * J;
			const float sc = lambda * 0.125f * emean * gd * (-2.f * J);
			y0 += sc * (ax ? ih[0] : -ih[0]);
			y1 += sc * (ay ? ih[1] : -ih[1]);
			y2 += sc * (az ? ih[2] : -ih[2]);
		}
	}
	// the node's row: sum over its eight elements (lanes 8g .. 8g + 7)
#pragma unroll
	for(int o = 1; o < 8; o <<= 1)
	{
		y0 += __shfl_xor_sync(0xffffffffu, y0, o);
		y1 += __shfl_xor_sync(0xffffffffu, y1, o);
		y2 += __shfl_xor_sync(0xffffffffu, y2, o);
	}
	if(node_ok && a == 0)
	{
		const int n = cg_node(L, x, y, z);
		const unsigned fl = cg_vflag(L, x, y, z);
		const float *bi = BI + 3 * (size_t)(L.coff[colour] + q);
		const float r[3] = {y0, y1, y2};
#pragma unroll
		for(int i = 0; i < 3; ++i)
			if(!((fl >> i) & 1u))
				d[3 * n + i] += (F[3 * n + i] - r[i]) * bi[i];
	}
}

__global__ void k_mf_eta32(int n, const double *__restrict__ evi, float *__restrict__ eta)
{
	pdl_begin();
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if(i < n)
		eta[i] = (float)evi[i];
}

template <typename... KArgs, typename... Args>
void mf_launch(void (*kern)(KArgs...), int blocks, int threads, cudaStream_t st, Args... args)
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

void launch_mf_eta32(cudaStream_t st, const Lvl &L, const double *evi, float *eta)
{
	const int n = 8 * L.nel;
	mf_launch(k_mf_eta32, (n + 255) / 256, 256, st, n, evi, eta);
}

void launch_mf_gs(cudaStream_t st, const Lvl &L, const float *eta, int aug, double lambda, const float *BI, const float *F,
                  float *d, int colour)
{
	const int n = L.coff[colour + 1] - L.coff[colour];
	if(n <= 0)
		return;
	const int blocks = (8 * n + MF_THREADS - 1) / MF_THREADS;
	if(aug)
		mf_launch(k_mf_gs<true>, blocks, MF_THREADS, st, L, eta, BI, F, d, colour, (float)lambda);
	else
		mf_launch(k_mf_gs<false>, blocks, MF_THREADS, st, L, eta, BI, F, d, colour, (float)lambda);
}
