// Allocation-free surface Nusselt numbers (heat_flux) for callers that must
// not allocate device memory.
//
// Who needs this: code that computes diagnostics from inside a host
// application that owns the whole device memory budget through its own pool
// (a coupled solver, an in-situ analysis hook, a framework whose allocator
// must see every byte), or code that is not allowed to call cudaMalloc at the
// point where it runs (for instance between the steps of someone else's
// captured work).  The regular path, citcom_gpu_heat_flux, needs a handle
// whose creation allocates every solver buffer; this entry point needs none.
//
// Its scratch (the per-element and nodal flux arrays, the reduction partials,
// the element geometry and the result) lives in one file-scope device array
// of fixed size, reserved when the library is loaded and held by every GPU
// that loads the library until the process exits.  All calls share it, so
// calls that overlap on the GPU (two host threads, or two streams) race on
// it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/citcom_gb300.h"
#include "kernels.h"

namespace {

constexpr int GEO_WORDS = (int)((sizeof(Geo) + sizeof(double) - 1) / sizeof(double));
constexpr int RED_WORDS = RED_MAX_BLOCKS * 8;
// layout (in doubles): geometry | reduction partials | counter + result | element means | nodal fluxes
constexpr long OFF_GEO = 0;
constexpr long OFF_RED = ((OFF_GEO + GEO_WORDS + 31) / 32) * 32;
constexpr long OFF_CTR = OFF_RED + RED_WORDS;  // one word for the counter
constexpr long OFF_OUT = OFF_CTR + 4;           // top and bottom flux sums, top and bottom weights
constexpr long OFF_WORK = ((OFF_OUT + 4 + 31) / 32) * 32;
constexpr long SCRATCH_WORDS = OFF_WORK + CITCOM_GPU_NOALLOC_MAX_ELEMENTS + CITCOM_GPU_NOALLOC_MAX_NODES;
constexpr int MAX_DEVICES = 64;

} // namespace

// the scratch: a fixed device array, no runtime allocation
static __device__ __align__(256) double g_noalloc_scratch[SCRATCH_WORDS];

namespace {

// device address of g_noalloc_scratch on each device, looked up once per
// device with that device current (the host-side symbol is not an address
// the GPU can use); the lock orders first calls made on several host threads
void *g_scratch_addr[MAX_DEVICES];
std::mutex g_scratch_lock;

int scratch_for_current_device(double **out)
{
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if(e != cudaSuccess || dev < 0 || dev >= MAX_DEVICES)
	{
		fprintf(stderr, "citcom_gpu_heat_flux_noalloc: no usable current device (%s)\n", cudaGetErrorString(e));
		return CITCOM_GPU_ERR_CUDA;
	}
	std::lock_guard<std::mutex> lock(g_scratch_lock);
	if(!g_scratch_addr[dev])
	{
		void *p = nullptr;
		e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if(e != cudaSuccess || !p)
		{
			fprintf(stderr, "citcom_gpu_heat_flux_noalloc: cudaGetSymbolAddress failed on device %d: %s\n", dev,
			        cudaGetErrorString(e));
			return CITCOM_GPU_ERR_CUDA;
		}
		g_scratch_addr[dev] = p;
	}
	*out = static_cast<double *>(g_scratch_addr[dev]);
	return CITCOM_GPU_OK;
}

void fill_level(Lvl &L, int nox, int noy, int noz, const double dimen[3])
{
	memset(&L, 0, sizeof(L));
	L.nox = nox;
	L.noy = noy;
	L.noz = noz;
	L.elx = nox - 1;
	L.ely = noy - 1;
	L.elz = noz - 1;
	L.nno = nox * noy * noz;
	L.nel = L.elx * L.ely * L.elz;
	L.neq = 3 * L.nno;
	L.npad = (L.nno + 31) / 32 * 32;
	L.h[0] = dimen[0] / L.elx;
	L.h[1] = dimen[1] / L.ely;
	L.h[2] = dimen[2] / L.elz;
	L.J = L.h[0] * L.h[1] * L.h[2] / 8.0;
}

} // namespace

extern "C" int citcom_gpu_heat_flux_noalloc(int nox, int noy, int noz, const double dimen[3], const double *dT, const double *dV,
                                            double *nut, double *nub)
{
	if(!dimen || !dT || !dV || nox < 2 || noy < 2 || noz < 2 || !(dimen[0] > 0.0 && dimen[1] > 0.0 && dimen[2] > 0.0))
	{
		fprintf(stderr, "citcom_gpu_heat_flux_noalloc: invalid arguments\n");
		return CITCOM_GPU_ERR_ARG;
	}
	const long nno = (long)nox * noy * noz;
	const long nel = (long)(nox - 1) * (noy - 1) * (noz - 1);
	if(nno > CITCOM_GPU_NOALLOC_MAX_NODES || nel > CITCOM_GPU_NOALLOC_MAX_ELEMENTS)
	{
		fprintf(stderr,
		        "citcom_gpu_heat_flux_noalloc: mesh of %ld nodes / %ld elements exceeds the fixed scratch of %d nodes / %d "
		        "elements; use citcom_gpu_heat_flux\n",
		        nno, nel, CITCOM_GPU_NOALLOC_MAX_NODES, CITCOM_GPU_NOALLOC_MAX_ELEMENTS);
		return CITCOM_GPU_ERR_ARG;
	}
	double *base = nullptr;
	int r = scratch_for_current_device(&base);
	if(r != CITCOM_GPU_OK)
		return r;

	Lvl L;
	fill_level(L, nox, noy, noz, dimen);
	Geo g;
	geo_fill_host(L, &g);
	Geo *dgeo = reinterpret_cast<Geo *>(base + OFF_GEO);
	Red red;
	red.partials = base + OFF_RED;
	red.counter = reinterpret_cast<unsigned *>(base + OFF_CTR);
	double *dout = base + OFF_OUT;
	double *work = base + OFF_WORK;

	// legacy default stream; the scratch keeps the previous call's contents,
	// so the reduction counter is cleared before use
	cudaStream_t st = 0;
	cudaError_t e = cudaMemcpyAsync(dgeo, &g, sizeof(Geo), cudaMemcpyHostToDevice, st);
	if(e == cudaSuccess)
		e = cudaMemsetAsync(red.counter, 0, sizeof(double), st);
	if(e == cudaSuccess)
	{
		launch_heat_flux(st, L, dgeo, dT, dV, work, red, dout);
		e = cudaGetLastError();
	}
	double sums[4] = {0.0, 0.0, 0.0, 0.0};
	if(e == cudaSuccess)
		e = cudaMemcpyAsync(sums, dout, sizeof(sums), cudaMemcpyDeviceToHost, st);
	if(e == cudaSuccess)
		e = cudaStreamSynchronize(st);
	if(e != cudaSuccess)
	{
		fprintf(stderr, "citcom_gpu_heat_flux_noalloc: %s\n", cudaGetErrorString(e));
		return CITCOM_GPU_ERR_CUDA;
	}
	if(nut)
		*nut = sums[0] / (4.0 * sums[2]);
	if(nub)
		*nub = sums[1] / (4.0 * sums[3]);
	return CITCOM_GPU_OK;
}
