// Host driver of the GB300 Stokes / SUPG path behind the C ABI of
// include/citcom_gb300.h.
//
// One handle owns every device buffer of one problem (allocated in
// citcom_gpu_create, nothing allocated afterwards) and one CUDA stream.  The
// Uzawa loop (solve_Ahat_p_fhat) and the solve_del2_u loop run on the host and
// read back a few scalars per iteration; one full-multigrid pass (multi_grid)
// is a fixed kernel sequence and is replayed as a captured CUDA graph.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/citcom_gb300.h"
#include "kernels.h"
#include "nn.h"

namespace {

enum Slot
{
	S_RES = 0,    // r.r of the solve_del2_u residual after a multigrid pass
	S_ERR = 1,    // set by the cluster program when one of its waits timed out
	S_LS = 2,     // line search (AU.res, AU.AU)
	S_R0 = 4,     // scratch dots
	S_DOT = 8,    // 4 dots
	S_NU = 32,    // heat flux: top and bottom sums, top and bottom weights
	S_VRMS = 36,  // sum of |u|^2 dV, volume
	S_MIN = 20,
	S_MAX = 21,
	S_UZ = 22,    // Uzawa scalars: r1.z1, r0.z0, s2.Ahat, alpha, error flag
	S_TERR = 31,  // (host mirror only) the tile kernels' error word
	S_COUNT = 40
};

template <typename T> struct MG
{
	T *vel[CITCOM_MAX_LEVELS], *res[CITCOM_MAX_LEVELS], *rhs[CITCOM_MAX_LEVELS], *fl[CITCOM_MAX_LEVELS],
		*del[CITCOM_MAX_LEVELS], *AU[CITCOM_MAX_LEVELS];
	T *K[CITCOM_MAX_LEVELS], *BI[CITCOM_MAX_LEVELS];
};

} // namespace

struct citcom_gpu
{
	citcom_gpu_config cfg;
	int L;
	Lvl lv[CITCOM_MAX_LEVELS];
	Geo *geo[CITCOM_MAX_LEVELS];
	double *evi[CITCOM_MAX_LEVELS];
	double *K64[CITCOM_MAX_LEVELS];
	double *BI64[CITCOM_MAX_LEVELS];
	float *K32[CITCOM_MAX_LEVELS];
	float *BI32[CITCOM_MAX_LEVELS];
	float4 *Kt32[CITCOM_MAX_LEVELS];  // padded FP32 stencil of the levels k_gs_tiny smooths, else null
	float *eta32[CITCOM_MAX_LEVELS];  // FP32 Gauss-point viscosity of the levels the matrix-free smoother relaxes, else null
	float *geodf[CITCOM_MAX_LEVELS];  // element kernels as FP32 pairs, word-major over the columns (mixed), else null
	float *K32lo;                     // mixed box: the finest FP64 operator's FP32 remainder (K64 = K32 + K32lo), else null
	float2 *usplit;                   // the vector K32 + K32lo is applied to, as FP32 pairs (neq)
	bool no_split;                    // CITCOM_GPU_NO_SPLIT: keep the finest FP64 stencil instead
	float2 *eta2[CITCOM_MAX_LEVELS];  // Gauss-point viscosity as FP32 pairs for the double-float assembly
	bool fp64_assembly;               // CITCOM_GPU_FP64_ASSEMBLY: the mixed configuration assembles in FP64
	double *BPI;
	MG<double> mg64;
	MG<float> mg32;
	double *visc_work[2];
	// fine-level fields
	double *U, *P, *F, *T, *Tdot, *V, *buoy;
	double *r0, *r1, *r2, *z0, *z1, *s1, *s2, *Ah, *u1;
	double *r64;           // FP64 residual of the refinement loop (mixed mode)
	double *Eres, *DTdot, *T1, *Tdot1, *hf_work;
	double *dscal;
	double *hscal;         // pinned mirror of dscal
	Red red;
	cudaStream_t st;
	cudaEvent_t ev0, ev1;
	cudaEvent_t ev_pass[2];  // brackets each multigrid pass
	cudaEvent_t ev_energy[2];  // brackets the PG_timestep of step_resident
	cudaEvent_t ev_asm[2];     // brackets the operator assembly of stokes_resident
	cudaEvent_t ev_gs[8];   // brackets the finest-level smoother calls inside a multigrid pass
	int n_gs_pairs;         // pairs recorded by the captured pass
	cudaGraphExec_t mg_exec;
	unsigned long long pass_kernels;   // kernels in one captured multigrid pass
	unsigned long long launches;       // kernels this handle has run
	bool stiffness_ready;
	bool visc_ready;
	bool verbose;
	double last_r0;  // the start residual of the last solve_del2_u (RMS per equation)
	bool no_graph;
	bool level_timing;            // CITCOM_GPU_LEVEL_TIMING: time every smoother call (no graph)
	bool no_tiny;                 // CITCOM_GPU_NO_TINY: coarsest FP32 levels use k_gs_small instead of k_gs_tiny
	bool mf;                      // matrix-free FP32 smoother on the large box levels (CITCOM_GPU_MF)
	// FP32 multigrid work of levels 0..co_LC runs as one cluster program per
	// stretch of consecutive coarse operations (co_LC = -1: off;
	// CITCOM_GPU_NO_CLUSTER disables it)
	int co_LC;
	int co_cluster;
	size_t co_smem;
	bool co_local[CITCOM_MAX_LEVELS];
	// the zero-start smoothing of level 0 as one dense product d = N f
	// (CITCOM_GPU_NO_DENSE keeps the sweeps): N and its build scratch
	float *co_dense;
	float *co_dense_work;
	// the same for level 1 (its sweeps of `co_dense1_cycles`, zero start or
	// with a start through d0 + N (f - K d0)) when it runs in the cluster program
	float *co_dense1;
	int co_dense1_cycles;
	CoLevels co_lv;
	CoProg co_prog;
	double lt_ms[CITCOM_MAX_LEVELS];
	long lt_calls[CITCOM_MAX_LEVELS];
	long lt_sweeps[CITCOM_MAX_LEVELS];
	citcom_gpu_stats stats;
	std::vector<void *> allocs;
	citcom_nn *warm;   // warm-start network attached to the Stokes solve (not owned), or null
	double diff_ts;    // diffusive time-step limit of the finest level
	double *oldU;      // the previous viscosity iteration's U (general_stokes_solver's oldU, kept across solves)
	double *T_sol;     // T of the last completed Stokes solve (the increment warm start's reference state)
	bool T_sol_valid;  // false until a solve completes after the last load_state
	unsigned state_gen;  // counts load_state calls (a new state sequence)
	double *edot;      // strain-rate invariant per fine element
	int sdepv_visits;  // calls of visc_from_S so far (the first one takes a unit strain rate)
	// output steps: device staging of the fields (allocated on first use), the
	// stream of their host copies, the event that orders it after the compute
	// stream and the event of its completion
	double *snap;
	cudaStream_t st_out;
	cudaEvent_t ev_snap, ev_out;
	bool snap_pending;
	char err[512];
};

// The warm-start network of one solver handle and its training set.
struct citcom_nn
{
	citcom_gpu *h;          // the solver (null once it is destroyed)
	NnNet *net;
	int lev, r;             // network level; node spacing ratio to the finest level
	int V;                  // network nodes
	int capacity, count, next;
	__nv_bfloat16 *xs;      // training inputs, capacity x V x 16
	float *ts;              // training targets, capacity x V x 4
	__nv_bfloat16 *x;       // inputs of the current state
	float *y;               // network output, V x 16
	double *Uv[CITCOM_MAX_LEVELS];  // guessed velocity on the levels lev .. finest - 1
	double *Ug, *Pg;        // guess on the finest level
	double *work;           // FP64 scratch of the input/target/guess kernels
	double su, sp, mp;      // output scales per unit anomaly RMS: velocity, pressure; pressure offset
	bool scaled;
	// increment mode (CITCOM_NN_INCREMENT): the state of the previous record
	// and the fine temperature increment
	int mode;
	double *Tp, *Up, *Pp, *dT;
	// the comparison with the resident start: every check_every-th guessed
	// solve; guesses so far, whether the network won the last comparison and
	// its initial residual then
	int check_every;
	long guesses;
	bool net_ok;
	double r_ref;
	bool have_prev;
	unsigned prev_gen;

	bool attached;
	unsigned long long rng;
	std::vector<void *> allocs;
	char err[512];
};

namespace {

int fail(citcom_gpu *h, int code, const char *fmt, ...)
{
	if(h)
	{
		va_list ap;
		va_start(ap, fmt);
		vsnprintf(h->err, sizeof(h->err), fmt, ap);
		va_end(ap);
	}
	return code;
}

#define CK(call)                                                                                                   \
	do                                                                                                             \
	{                                                                                                              \
		cudaError_t e_ = (call);                                                                                   \
		if(e_ != cudaSuccess)                                                                                      \
			return fail(h, CITCOM_GPU_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
	} while(0)

#define TRY(call)               \
	do                          \
	{                           \
		int r_ = (call);        \
		if(r_ != CITCOM_GPU_OK) \
			return r_;          \
	} while(0)

template <typename T> int dalloc(citcom_gpu *h, T **p, size_t n)
{
	void *q = nullptr;
	cudaError_t e = cudaMalloc(&q, (n ? n : 1) * sizeof(T));
	if(e != cudaSuccess)
		return fail(h, CITCOM_GPU_ERR_CUDA, "cudaMalloc of %zu bytes: %s", n * sizeof(T), cudaGetErrorString(e));
	cudaMemset(q, 0, (n ? n : 1) * sizeof(T));
	h->allocs.push_back(q);
	*p = (T *)q;
	return CITCOM_GPU_OK;
}

void make_level(const citcom_gpu_config &c, int l, Lvl &L)
{
	memset(&L, 0, sizeof(L));
	L.nox = c.mgunit[0] * (1 << l) + 1;
	L.noy = c.mgunit[1] * (1 << l) + 1;
	L.noz = c.mgunit[2] * (1 << l) + 1;
	L.elx = L.nox - 1;
	L.ely = L.noy - 1;
	L.elz = L.noz - 1;
	L.nno = L.nox * L.noy * L.noz;
	L.nel = L.elx * L.ely * L.elz;
	L.neq = 3 * L.nno;
	L.npad = (L.nno + 31) / 32 * 32;
	L.aos = L.nno <= CG_SMALL_LEVEL_NODES;
	const int N[3] = {L.nox, L.noy, L.noz};
	for(int a = 0; a < 3; ++a)
		for(int p = 0; p < 2; ++p)
			L.cnt[a][p] = (N[a] - p + 1) / 2;
	cg_set_offsets(L);
	if(c.sphere)
	{
		// uniform theta, phi, r grid (Nodal_mesh.c:87-95, 202-217), angles in radians
		const double rad = M_PI / 180.0;
		L.sphere = 1;
		L.org[0] = c.theta[0] * rad;
		L.org[1] = c.fi[0] * rad;
		L.org[2] = c.radius[0];
		L.h[0] = (c.theta[1] - c.theta[0]) * rad / L.elx;
		L.h[1] = (c.fi[1] - c.fi[0]) * rad / L.ely;
		L.h[2] = (c.radius[1] - c.radius[0]) / L.elz;
		L.J = 0.0;
		return;
	}
	L.h[0] = c.dimen[0] / L.elx;
	L.h[1] = c.dimen[1] / L.ely;
	L.h[2] = c.dimen[2] / L.elz;
	L.J = L.h[0] * L.h[1] * L.h[2] / 8.0;
}

// L2 residency of the tile-major stencils (level.h: l2hint, l2keep).  A
// colour sweep streams its slice of the stencil once, so plain LRU keeps
// nothing of a level larger than the L2 from one sweep to the next.  The
// finest level is read a few times per pass and streams with evict_first;
// the coarser tile-major levels, smoothed many times per pass, keep a share
// with evict_last, from the coarsest up, until CITCOM_GPU_L2KEEP_MB (default
// 64 MB of the 129 MB L2; the rest holds the vectors) is spent.
// CITCOM_GPU_L2HINT=0 issues the copies without hints.
void set_l2_policy(citcom_gpu *h)
{
	const char *e = getenv("CITCOM_GPU_L2HINT");
	const bool on = !(e && e[0] == '0');
	const char *m = getenv("CITCOM_GPU_L2KEEP_MB");
	double budget = 1e6 * ((m && m[0]) ? atof(m) : 64.0);
	const int lmax = h->L - 1;
	const double word = h->cfg.precision == CITCOM_GPU_FP64 ? 8.0 : 4.0;
	for(int l = 0; l <= lmax; ++l)
	{
		Lvl &L = h->lv[l];
		L.l2hint = 0;
		L.l2keep = 0;
		// small levels and those of the cluster program are not tile-streamed
		if(!on || L.aos || l <= h->co_LC)
			continue;
		L.l2hint = 1;
		if(l == lmax)
			continue;
		const double bytes = word * (double)cg_kwords(L);
		const double frac = std::min(1.0, std::max(0.0, budget / bytes));
		L.l2keep = (int)(1000.0 * frac);
		budget -= frac * bytes;
	}
}

Red red_of(citcom_gpu *h) { return h->red; }

int readback(citcom_gpu *h, int slot, int n)
{
	CK(cudaMemcpyAsync(h->hscal + slot, h->dscal + slot, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
	CK(cudaStreamSynchronize(h->st));
	return CITCOM_GPU_OK;
}

// K u and f - K u with the finest level's FP64 operator: the FP64 stencil,
// or (mixed box) the FP32 pair K32 + K32lo in double-float arithmetic
void fine_kmul64(citcom_gpu *h, const double *u, double *out)
{
	const int lmax = h->L - 1;
	if(h->K32lo)
		launch_tile_split(h->st, h->lv[lmax], h->K32[lmax], h->K32lo, nullptr, u, h->usplit, out);
	else
		launch_kmul<double>(h->st, h->lv[lmax], h->K64[lmax], u, out);
}

void fine_residual64(citcom_gpu *h, const double *f, const double *u, double *r)
{
	const int lmax = h->L - 1;
	if(h->K32lo)
		launch_tile_split(h->st, h->lv[lmax], h->K32[lmax], h->K32lo, f, u, h->usplit, r);
	else
		launch_residual<double>(h->st, h->lv[lmax], h->K64[lmax], f, u, r);
}

// The error words of the kernels' bounded waits (the tile kernels' g_tile_err,
// the cluster program's dscal[S_ERR]) to zero, on the stream.
int device_errors_reset(citcom_gpu *h)
{
	if(tile_error_reset_async(h->st) != 0)
		return fail(h, CITCOM_GPU_ERR_CUDA, "clearing the tile kernels' error word failed");
	CK(cudaMemsetAsync(h->dscal + S_ERR, 0, sizeof(double), h->st));
	return CITCOM_GPU_OK;
}

// After h->hscal[S_TERR] and [S_ERR] were read back: CITCOM_GPU_ERR_CUDA with
// the reason when a bounded wait ran out (the words are cleared again, so the
// next call starts clean), else OK.
int device_errors_report(citcom_gpu *h, const char *where)
{
	const bool tile = h->hscal[S_TERR] != 0.0, clus = h->hscal[S_ERR] != 0.0;
	if(!tile && !clus)
		return CITCOM_GPU_OK;
	h->hscal[S_TERR] = h->hscal[S_ERR] = 0.0;
	device_errors_reset(h);
	cudaStreamSynchronize(h->st);
	return fail(h, CITCOM_GPU_ERR_CUDA, "%s: %s", where,
	            tile ? "a stencil tile copy did not arrive (a bounded wait ran out)"
	                 : "a wait of the cluster smoother timed out");
}

// reads both error words (synchronises) and reports as above
int device_errors_check(citcom_gpu *h, const char *where)
{
	if(tile_error_async(h->hscal + S_TERR, h->st) != 0)
		return fail(h, CITCOM_GPU_ERR_CUDA, "%s: reading the tile kernels' error word failed", where);
	TRY(readback(h, S_ERR, 1));
	return device_errors_report(h, where);
}

Rheo rheo_of(const citcom_gpu_config &c)
{
	Rheo r;
	memset(&r, 0, sizeof(r));
	r.tdepv = c.tdepv;
	r.num_mat = c.num_mat < 1 ? 1 : (c.num_mat > 8 ? 8 : c.num_mat);
	for(int i = 0; i < 8; ++i)
	{
		r.visc0[i] = c.visc0[i];
		r.viscE[i] = c.viscE[i];
		r.viscT[i] = c.viscT[i];
		r.z_layer[i] = c.z_layer[i];
	}
	r.vmin_on = c.vmin_on;
	r.vmax_on = c.vmax_on;
	r.vmin = c.vmin;
	r.vmax = c.vmax;
	r.sdepv = c.sdepv;
	r.sdepv_rheology = c.sdepv_rheology;
	for(int i = 0; i < 8; ++i)
	{
		r.sdepv_expt[i] = c.sdepv_expt[i];
		r.sdepv_trns[i] = c.sdepv_trns[i];
	}
	return r;
}

// ---------------------------------------------------------------- gauss_seidel

template <typename T> void gs_inner(citcom_gpu *h, MG<T> &B, int lev, T *d, const T *F, int cycles, int zero_start);

// Gauss-Seidel call; on the finest level the call is bracketed by timing
// events (captured into the multigrid graph) so that the dominant kernel's
// device time is measured live during every solve.
// vector `id` (CoVec) of level lev
template <typename T> T *mg_vec(MG<T> &B, int lev, int id)
{
	switch(id)
	{
	case CO_VEL: return B.vel[lev];
	case CO_DEL: return B.del[lev];
	case CO_RHS: return B.rhs[lev];
	case CO_RES: return B.res[lev];
	case CO_FL: return B.fl[lev];
	default: return B.AU[lev];
	}
}

// queued coarse operations run as one cluster program
void co_flush(citcom_gpu *h)
{
	if(h->co_prog.n > 0)
	{
		launch_coarse(h->st, h->co_lv, h->co_prog, h->co_cluster, h->co_smem);
		h->co_prog.n = 0;
	}
}

template <typename T> bool co_level(citcom_gpu *h, int lev)
{
	return std::is_same<T, float>::value && lev <= h->co_LC;
}

void co_push(citcom_gpu *h, int type, int lev, int a, int b, int c, int cycles = 0, int zero = 0)
{
	if(type == CO_GS && lev == 1 && h->co_dense1 && cycles == h->co_dense1_cycles)
	{
		// level 1's sweeps as its dense smoother matrix: d = N f from a zero
		// start, else AU = f - K d, then d += N AU (AU is free here: the line
		// search that follows a smoothing call recomputes it)
		if(!zero)
			co_push(h, CO_RESID, lev, b, a, CO_AU);
		co_push(h, CO_DENSE, lev, a, zero ? b : CO_AU, 0, cycles, zero);
		return;
	}
	if(h->co_prog.n == CO_MAX_OPS)
		co_flush(h);
	CoOp &op = h->co_prog.op[h->co_prog.n++];
	op.type = (unsigned char)type;
	op.lev = (unsigned char)lev;
	op.a = (unsigned char)a;
	op.b = (unsigned char)b;
	op.c = (unsigned char)c;
	op.zero = (unsigned char)zero;
	op.local = (unsigned char)(type == CO_GS && h->co_local[lev]);
	if(type == CO_GS && lev == 0 && zero && h->co_dense && cycles == h->cfg.vlowstep)
		op.type = CO_DENSE;
	op.pad = 0;
	op.cycles = (unsigned short)cycles;
}

template <typename T> void gs(citcom_gpu *h, MG<T> &B, int lev, T *d, const T *F, int cycles, int zero_start)
{
	const bool timed = (lev == h->L - 1) && h->n_gs_pairs < 4 && !gs_small_fits(h->lv[lev], sizeof(T));
	// during stream capture, external records become event-record nodes of
	// the graph; outside capture they are ordinary records
	unsigned flags = 0;
	if(timed)
	{
		cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
		cudaStreamIsCapturing(h->st, &cs);
		flags = (cs == cudaStreamCaptureStatusActive) ? cudaEventRecordExternal : 0u;
		cudaEventRecordWithFlags(h->ev_gs[2 * h->n_gs_pairs], h->st, flags);
	}
	if(h->level_timing)
	{
		cudaEventRecord(h->ev_gs[4], h->st);
		gs_inner<T>(h, B, lev, d, F, cycles, zero_start);
		cudaEventRecord(h->ev_gs[5], h->st);
		cudaEventSynchronize(h->ev_gs[5]);
		float ms = 0.f;
		cudaEventElapsedTime(&ms, h->ev_gs[4], h->ev_gs[5]);
		h->lt_ms[lev] += ms;
		h->lt_calls[lev] += 1;
		h->lt_sweeps[lev] += cycles;
	}
	else
		gs_inner<T>(h, B, lev, d, F, cycles, zero_start);
	if(timed)
	{
		cudaEventRecordWithFlags(h->ev_gs[2 * h->n_gs_pairs + 1], h->st, flags);
		h->n_gs_pairs++;
	}
}

template <typename T> void gs_inner(citcom_gpu *h, MG<T> &B, int lev, T *d, const T *F, int cycles, int zero_start)
{
	const Lvl &L = h->lv[lev];
	if constexpr(std::is_same<T, float>::value)
	{
		if(h->Kt32[lev] && !h->no_tiny)
		{
			launch_gs_tiny(h->st, L, h->Kt32[lev], B.BI[lev], F, d, cycles, zero_start);
			return;
		}
		if(h->eta32[lev])
		{
			// matrix-free colours (mf.cu) instead of the stored stencil
			if(zero_start)
				cudaMemsetAsync(d, 0, sizeof(T) * L.neq, h->st);
			for(int c = 0; c < cycles; ++c)
				for(int col = 0; col < 8; ++col)
					launch_mf_gs(h->st, L, h->eta32[lev], h->cfg.aug_lagr, h->cfg.aug_number, B.BI[lev], F, d, col);
			return;
		}
	}
	if(gs_small_fits(L, sizeof(T)))
	{
		launch_gs_small<T>(h->st, L, B.K[lev], B.BI[lev], F, d, cycles, zero_start);
		return;
	}
	if(zero_start)
		cudaMemsetAsync(d, 0, sizeof(T) * L.neq, h->st);
	for(int c = 0; c < cycles; ++c)
		for(int col = 0; col < 8; ++col)
			launch_gs_colour<T>(h->st, L, B.K[lev], B.BI[lev], F, d, col);
}

// ---------------------------------------------------------------- multi_grid

// The operations of a pass, by level and vector id: levels 0..co_LC of the
// FP32 solver are queued for the cluster program, the others launched at once
// (after the queue is flushed, so the order of the pass is kept).
template <typename T> void mg_gs(citcom_gpu *h, MG<T> &B, int lev, int d, int f, int cycles, int zero)
{
	if(!co_level<T>(h, lev))
	{
		co_flush(h);
		gs<T>(h, B, lev, mg_vec(B, lev, d), mg_vec(B, lev, f), cycles, zero);
		return;
	}
	if(!h->level_timing)
	{
		co_push(h, CO_GS, lev, d, f, 0, cycles, zero);
		return;
	}
	co_flush(h);
	cudaEventRecord(h->ev_gs[4], h->st);
	co_push(h, CO_GS, lev, d, f, 0, cycles, zero);
	co_flush(h);
	cudaEventRecord(h->ev_gs[5], h->st);
	cudaEventSynchronize(h->ev_gs[5]);
	float ms = 0.f;
	cudaEventElapsedTime(&ms, h->ev_gs[4], h->ev_gs[5]);
	h->lt_ms[lev] += ms;
	h->lt_calls[lev] += 1;
	h->lt_sweeps[lev] += cycles;
}

// vec r = vec f - K vec d
template <typename T> void mg_res(citcom_gpu *h, MG<T> &B, int lev, int f, int d, int r)
{
	if(co_level<T>(h, lev))
		return co_push(h, CO_RESID, lev, f, d, r);
	co_flush(h);
	launch_residual<T>(h->st, h->lv[lev], B.K[lev], mg_vec(B, lev, f), mg_vec(B, lev, d), mg_vec(B, lev, r));
}

// vec dst (level lev-1) = projection of vec src (level lev)
template <typename T> void mg_proj(citcom_gpu *h, MG<T> &B, int lev, int src, int dst)
{
	if(co_level<T>(h, lev))
		return co_push(h, CO_PROJ, lev, src, dst, 0);
	co_flush(h);
	launch_project<T>(h->st, h->lv[lev], h->lv[lev - 1], h->geo[lev - 1], mg_vec(B, lev, src), mg_vec(B, lev - 1, dst));
}

// vec dst (level lev) = interpolation of vec src (level lev-1)
template <typename T> void mg_interp(citcom_gpu *h, MG<T> &B, int lev, int src, int dst)
{
	if(co_level<T>(h, lev))
		return co_push(h, CO_INTERP, lev, src, dst, 0);
	co_flush(h);
	launch_interp<T>(h->st, h->lv[lev - 1], h->lv[lev], h->geo[lev], mg_vec(B, lev - 1, src), mg_vec(B, lev, dst));
}

// line search of the upward leg: AU = K del, vel += (AU.res / AU.AU) del
// (and res -= alpha AU on the finest level)
template <typename T> void mg_linesearch(citcom_gpu *h, MG<T> &B, int lev, bool finest)
{
	if(co_level<T>(h, lev) && !finest)
	{
		co_push(h, CO_KDOT, lev, CO_DEL, CO_RES, CO_AU, 0, 1);  // with the update vel += alpha del
		return;
	}
	co_flush(h);
	const Lvl &L = h->lv[lev];
	launch_kmul_linesearch<T>(h->st, L, B.K[lev], B.del[lev], B.res[lev], B.AU[lev], red_of(h), h->dscal + S_LS);
	launch_vel_update<T>(h->st, L.neq, B.vel[lev], B.del[lev], B.res[lev], B.AU[lev], h->dscal + S_LS, finest);
}

// One full-multigrid pass (multi_grid, General_matrix_functions.c:525-653).
// Input: fl[lmax].  Output: vel[lmax] (the correction) and res[lmax].
template <typename T> void mg_pass(citcom_gpu *h, MG<T> &B)
{
	const citcom_gpu_config &c = h->cfg;
	const int lmax = h->L - 1, lmin = 0;
	for(int lev = lmax; lev > lmin; --lev)
		mg_proj<T>(h, B, lev, CO_FL, CO_FL);
	mg_gs<T>(h, B, lmin, CO_VEL, CO_FL, c.vlowstep, 1);
	for(int lev = lmin + 1; lev <= lmax; ++lev)
	{
		mg_interp<T>(h, B, lev, CO_VEL, CO_VEL);
		for(int Vn = 1; Vn <= c.mg_cycle; ++Vn)
		{
			for(int dlev = lev; dlev >= lmin + 1; --dlev)
			{
				const int cyc = (dlev == lmax) ? c.vhighstep : c.down_heavy;
				const int rhs = (dlev == lev) ? CO_FL : CO_RHS;
				mg_gs<T>(h, B, dlev, CO_VEL, rhs, cyc, dlev != lev);
				mg_res<T>(h, B, dlev, rhs, CO_VEL, CO_RES);
				mg_proj<T>(h, B, dlev, CO_RES, CO_RHS);
			}
			mg_gs<T>(h, B, lmin, CO_VEL, CO_RHS, c.vlowstep, 1);
			for(int ulev = lmin + 1; ulev <= lev; ++ulev)
			{
				const int cyc = (ulev == lmax) ? c.vhighstep : c.up_heavy;
				mg_interp<T>(h, B, ulev, CO_VEL, CO_DEL);
				mg_gs<T>(h, B, ulev, CO_DEL, CO_RES, cyc, 0);
				mg_linesearch<T>(h, B, ulev, ulev == lmax);
			}
		}
	}
	co_flush(h);
}

// the pass plus solve_del2_u's bookkeeping; FP64: r (= fl[lmax]) <- res, d0 += vel;
// mixed: FP32 pass on (float) r, d0 += vel, r = F - K64 d0 in FP64
int record_pass(citcom_gpu *h)
{
	const Lvl &Lf = h->lv[h->L - 1];
	const int lmax = h->L - 1;
	if(h->cfg.precision == CITCOM_GPU_FP64)
	{
		mg_pass<double>(h, h->mg64);
		launch_axpby(h->st, Lf.neq, h->u1, 1.0, h->mg64.vel[lmax], 1.0);
		CK(cudaMemcpyAsync(h->mg64.fl[lmax], h->mg64.res[lmax], sizeof(double) * Lf.neq, cudaMemcpyDeviceToDevice, h->st));
		launch_dot(h->st, Lf.neq, h->mg64.res[lmax], h->mg64.res[lmax], red_of(h), h->dscal + S_RES);
	}
	else
	{
		launch_copy_d2f(h->st, Lf.neq, h->mg32.fl[lmax], h->r64);
		mg_pass<float>(h, h->mg32);
		launch_add_f2d(h->st, Lf.neq, h->u1, h->mg32.vel[lmax]);
		fine_residual64(h, h->Ah, h->u1, h->r64);
		launch_dot(h->st, Lf.neq, h->r64, h->r64, red_of(h), h->dscal + S_RES);
	}
	return CITCOM_GPU_OK;
}

int run_pass(citcom_gpu *h)
{
	if(h->no_graph)
	{
		// direct launches (for kernel profilers that do not follow graphs)
		h->n_gs_pairs = 0;
		TRY(record_pass(h));
		CK(cudaGetLastError());
		return CITCOM_GPU_OK;
	}
	if(!h->mg_exec)
	{
		cudaGraph_t g;
		h->n_gs_pairs = 0;
		const unsigned long long k0 = g_kernel_launches;
		CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
		int r = record_pass(h);
		cudaError_t e = cudaStreamEndCapture(h->st, &g);
		h->pass_kernels = g_kernel_launches - k0;
		g_kernel_launches = k0;
		if(r != CITCOM_GPU_OK)
			return r;
		CK(e);
		CK(cudaGraphInstantiate(&h->mg_exec, g, 0));
		CK(cudaGraphDestroy(g));
	}
	CK(cudaGraphLaunch(h->mg_exec, h->st));
	g_kernel_launches += h->pass_kernels;
	return CITCOM_GPU_OK;
}

// solve_del2_u (General_matrix_functions.c:368-520) for K d0 = F with
// d0 = h->u1 and F = h->Ah (the only pair the Uzawa solver passes).
int solve_del2_u(citcom_gpu *h, double acc, int *valid)
{
	const Lvl &Lf = h->lv[h->L - 1];
	const int neq = Lf.neq;
	double *r = (h->cfg.precision == CITCOM_GPU_FP64) ? h->mg64.fl[h->L - 1] : h->r64;
	CK(cudaMemcpyAsync(r, h->Ah, sizeof(double) * neq, cudaMemcpyDeviceToDevice, h->st));
	CK(cudaMemsetAsync(h->u1, 0, sizeof(double) * (neq + 2), h->st));
	launch_dot(h->st, neq, r, r, red_of(h), h->dscal + S_RES);
	TRY(readback(h, S_RES, 2));
	const double r0 = std::sqrt(h->hscal[S_RES] / neq);
	h->last_r0 = r0;
	double residual = r0;
	if(r0 * h->cfg.accuracy > acc)
		acc = r0 * h->cfg.accuracy;
	*valid = (residual < acc) ? 0 : 1;
	int count = 0;
	while(residual > acc)
	{
		if(count >= 1000)
			return fail(h, CITCOM_GPU_ERR_NOCONV, "solve_del2_u: no convergence after %d multigrid passes (residual %g > %g)",
			            count, residual, acc);
		CK(cudaEventRecord(h->ev_pass[0], h->st));
		TRY(run_pass(h));
		CK(cudaEventRecord(h->ev_pass[1], h->st));
		if(tile_error_async(h->hscal + S_TERR, h->st) != 0)
			return fail(h, CITCOM_GPU_ERR_CUDA, "solve_del2_u: reading the tile kernels' error word failed");
		TRY(readback(h, S_RES, 2));
		TRY(device_errors_report(h, "solve_del2_u"));
		residual = std::sqrt(h->hscal[S_RES] / neq);
		{
			float ms = 0.f;
			if(cudaEventElapsedTime(&ms, h->ev_pass[0], h->ev_pass[1]) == cudaSuccess)
				h->stats.pass_ms += ms;
			else
				cudaGetLastError();
		}
		for(int k = 0; k < h->n_gs_pairs; ++k)
		{
			float ms = 0.f;
			if(cudaEventElapsedTime(&ms, h->ev_gs[2 * k], h->ev_gs[2 * k + 1]) == cudaSuccess)
			{
				h->stats.smoother_ms += ms;
				h->stats.smoother_sweeps += h->cfg.vhighstep;
			}
			else
				cudaGetLastError();
		}
		if(!(residual == residual))
			return fail(h, CITCOM_GPU_ERR_NOCONV, "solve_del2_u: residual is NaN");
		++count;
	}
	h->stats.mg_passes += count;
	h->stats.del2_calls += 1;
	return CITCOM_GPU_OK;
}

// ---------------------------------------------------------------- Uzawa

int nn_guess(citcom_nn *n);
int nn_increment_guess(citcom_nn *n, const double *V, const double *P);

// The head of solve_Ahat_p_fhat (Stokes_flow_Incomp.c:360-371): the velocity
// correction V += K^-1 (F - G P - K V) for the pressure P, then r1 = B V and
// the initial residual |r1| / sqrt(npno) that the function returns.  With
// vv != null also V.V (the residual rule's continuity test needs it).
int uzawa_start(citcom_gpu *h, double *V, const double *P, const double *F, double acc, double *r1, double *residual,
                double *vv = nullptr)
{
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	const Geo *geo = h->geo[lmax];
	cudaStream_t st = h->st;
	int valid;
	launch_grad(st, Lf, geo, P, h->Ah);
	fine_kmul64(h, V, h->u1);
	launch_sub3(st, Lf.neq, h->Ah, F, h->Ah, h->u1);
	launch_strip(st, Lf, h->Ah);
	const int passes0 = h->stats.mg_passes;
	TRY(solve_del2_u(h, acc, &valid));
	if(h->verbose)
		fprintf(stderr, "AhatP head: |F - GP - KV| %9.3e, %d multigrid passes to %9.3e\n", h->last_r0,
		        h->stats.mg_passes - passes0, acc);
	launch_strip(st, Lf, h->u1);
	launch_axpby(st, Lf.neq, V, 1.0, h->u1, 1.0);
	launch_div(st, Lf, geo, V, r1);
	launch_dot(st, Lf.nel, r1, r1, red_of(h), h->dscal + S_R0);
	if(vv)
		launch_dot(st, Lf.neq, V, V, red_of(h), h->dscal + S_R0 + 1);
	TRY(readback(h, S_R0, vv ? 2 : 1));
	*residual = std::sqrt(h->hscal[S_R0] / Lf.nel);
	if(vv)
		*vv = h->hscal[S_R0 + 1];
	return CITCOM_GPU_OK;
}

// |F - K V - G P|^2 with the FP64 operator of the finest level (constrained
// rows are zero in F, G P and K V alike)
int momentum_rr(citcom_gpu *h, const double *V, const double *P, const double *F, double *rr)
{
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	launch_grad(h->st, Lf, h->geo[lmax], P, h->Ah);
	fine_kmul64(h, V, h->u1);
	launch_sub3(h->st, Lf.neq, h->r64, F, h->Ah, h->u1);
	launch_dot(h->st, Lf.neq, h->r64, h->r64, red_of(h), h->dscal + S_R0 + 2);
	TRY(readback(h, S_R0 + 2, 1));
	*rr = h->hscal[S_R0 + 2];
	return CITCOM_GPU_OK;
}

// continuity residual of the residual rule: |B V| / (|V| sqrt(npno/neq))
double continuity(double bvbv, double vv, int neq, int npno)
{
	return std::sqrt(bvbv / (vv > 0.0 ? vv : 1e-300) * ((double)neq / (double)npno));
}

// solve_Ahat_p_fhat (Stokes_flow_Incomp.c:295-497) on device buffers.  With a
// warm-start network attached, the head runs for the network's guess as well
// as for the given V, P, and the loop continues from the pair with the smaller
// initial residual.  Stopping: the reference's rule (dv/v, dp/p) or the
// residual rule of citcom_gpu_config.stop_rule.
int uzawa(citcom_gpu *h, double *V, double *P, const double *F, double imp, int *steps_max, double *initial_residual)
{
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	const int neq = Lf.neq, npno = Lf.nel;
	const Geo *geo = h->geo[lmax];
	cudaStream_t st = h->st;
	double *Ah = h->Ah, *u1 = h->u1;
	const bool resid_rule = h->cfg.stop_rule == CITCOM_GPU_STOP_RESIDUAL;
	int valid;
	if(!h->stiffness_ready)
		return fail(h, CITCOM_GPU_ERR_STATE, "construct_stiffness_B_matrix has not been called");

	// F.F, and the error words of the kernels since the last check (operator
	// assembly: the coarsest level's dense smoother is built by the cluster
	// program's smoother)
	launch_dot(st, neq, F, F, red_of(h), h->dscal + S_R0);
	if(tile_error_async(h->hscal + S_TERR, st) != 0)
		return fail(h, CITCOM_GPU_ERR_CUDA, "solve_Ahat_p_fhat: reading the tile kernels' error word failed");
	TRY(readback(h, 0, S_R0 + 1));
	TRY(device_errors_report(h, "solve_Ahat_p_fhat"));
	const double ff = h->hscal[S_R0];
	const double v_res = std::sqrt(ff / neq);

	h->stats.warm_start = 0;
	h->stats.warm_residual = 0.0;
	h->stats.base_residual = 0.0;
	h->stats.corrections = 0;
	h->stats.final_momentum = 0.0;
	h->stats.final_continuity = 0.0;
	double residual = 0.0, vv = 0.0;
	double *vvp = resid_rule ? &vv : nullptr;
	citcom_nn *n = h->warm;
	// increment mode: a guess exists once a solve of the same state sequence
	// has completed (T_sol is its temperature)
	const bool inc = n && n->scaled && n->mode == CITCOM_NN_INCREMENT;
	h->stats.warm_compared = 0;
	if(n && n->scaled && (!inc || h->T_sol_valid))
	{
		// The network's start is compared with the resident one (both heads
		// run, the smaller initial residual wins) on every check_every-th
		// guessed solve, and whenever the guess's initial residual has grown
		// past 4x that of the last comparison the network won.  Between
		// comparisons the last winner is used alone.
		const bool scheduled = n->check_every <= 1 || n->guesses % n->check_every == 0;
		n->guesses++;
		if(!scheduled && !n->net_ok)
			TRY(uzawa_start(h, V, P, F, imp * v_res, h->r1, &residual, vvp));
		else
		{
			double r_net = 0.0, vv_net = 0.0;
			if(inc)
				TRY(nn_increment_guess(n, V, P));
			else
				TRY(nn_guess(n));
			TRY(uzawa_start(h, n->Ug, n->Pg, F, imp * v_res, h->r1, &r_net, resid_rule ? &vv_net : nullptr));
			const bool compare = scheduled || !(r_net <= 4.0 * n->r_ref);
			residual = HUGE_VAL;
			if(compare)
				TRY(uzawa_start(h, V, P, F, imp * v_res, h->r1, &residual, vvp));
			if(nn_device_error(n->net) != 0)
				return fail(h, CITCOM_GPU_ERR_CUDA, "warm-start network: a tensor-core wait timed out");
			h->stats.warm_compared = compare ? 1 : 0;
			h->stats.warm_residual = r_net;
			h->stats.base_residual = compare ? residual : 0.0;
			if(r_net < residual)
			{
				CK(cudaMemcpyAsync(V, n->Ug, sizeof(double) * neq, cudaMemcpyDeviceToDevice, st));
				CK(cudaMemcpyAsync(P, n->Pg, sizeof(double) * npno, cudaMemcpyDeviceToDevice, st));
				launch_div(st, Lf, geo, V, h->r1);
				residual = r_net;
				vv = vv_net;
				h->stats.warm_start = 1;
				if(compare)
				{
					n->net_ok = true;
					n->r_ref = r_net;
				}
			}
			else
				n->net_ok = false;
		}
	}
	else
		TRY(uzawa_start(h, V, P, F, imp * v_res, h->r1, &residual, vvp));
	double *r0 = h->r0, *r1 = h->r1, *r2 = h->r2, *z0 = h->z0, *z1 = h->z1, *s1 = h->s1, *s2 = h->s2, *sh;

	int count = 0;
	double dpressure = 1.0, dvelocity = 1.0;
	// residual rule: continuity of the current V (from r1 = B V) and whether
	// the next iteration starts a new search direction
	double cont = resid_rule ? continuity(residual * residual * npno, vv, neq, npno) : 0.0;
	bool restart = true;
	double *sc = h->dscal + S_UZ;
	CK(cudaMemsetAsync(sc, 0, 5 * sizeof(double), st));
	for(;;)
	{
		if(resid_rule)
		{
			if(cont <= imp)
			{
				double rr = 0.0;
				TRY(momentum_rr(h, V, P, F, &rr));
				const double mom = std::sqrt(rr / (ff > 0.0 ? ff : 1.0));
				h->stats.final_momentum = mom;
				h->stats.final_continuity = cont;
				if(h->verbose)
					fprintf(stderr, "AhatP check after %d iterations: continuity %9.3e momentum %9.3e\n", count, cont, mom);
				if(mom <= imp || h->stats.corrections >= 8)
					break;
				// velocity correction to half the tolerance, then B V afresh
				double rc = 0.0;
				TRY(uzawa_start(h, V, P, F, 0.5 * imp * v_res, r1, &rc, &vv));
				h->stats.corrections++;
				cont = continuity(rc * rc * npno, vv, neq, npno);
				h->stats.final_continuity = cont;
				restart = true;
				if(h->verbose)
					fprintf(stderr, "AhatP correction %d: momentum %9.3e -> continuity %9.3e\n", h->stats.corrections, mom,
					        cont);
				continue;
			}
			if(count >= *steps_max)
				break;
		}
		else if(!(count < *steps_max && (dpressure >= imp || dvelocity >= imp)))
			break;
		// z1 = BPI r1, r1.z1, search direction s2 (scalars stay on the device)
		launch_uzawa_precond(st, npno, h->BPI, r1, z1, red_of(h), sc);
		launch_uzawa_search(st, npno, s2, z1, s1, sc, restart);
		restart = false;
		launch_grad(st, Lf, geo, s2, Ah);
		TRY(solve_del2_u(h, imp * v_res, &valid));
		launch_strip(st, Lf, u1);
		launch_div(st, Lf, geo, u1, Ah);
		launch_dot(st, npno, s2, Ah, red_of(h), sc + 2);
		launch_uzawa_update(st, npno, neq, r2, r1, Ah, P, s2, V, u1, sc, valid);
		launch_dots4(st, neq, V, V, u1, u1, nullptr, nullptr, nullptr, nullptr, red_of(h), h->dscal + S_DOT);
		launch_dots4(st, npno, P, P, s2, s2, r2, r2, nullptr, nullptr, red_of(h), h->dscal + S_DOT + 4);
		CK(cudaMemcpyAsync(h->hscal + S_DOT, h->dscal + S_DOT, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
		TRY(readback(h, S_UZ, 5));
		if(h->hscal[S_UZ + 4] != 0.0)
			return fail(h, CITCOM_GPU_ERR_NOCONV, "solve_Ahat_p_fhat: division by zero in head of incompressibility iteration");
		const double alpha = h->hscal[S_UZ + 3];
		const double vdotv = h->hscal[S_DOT], u1u1 = h->hscal[S_DOT + 1];
		const double pdotp = h->hscal[S_DOT + 4], s2s2 = h->hscal[S_DOT + 5], r2r2 = h->hscal[S_DOT + 6];
		dpressure = alpha * std::sqrt(s2s2 / (1.0e-32 + pdotp));
		dvelocity = alpha * std::sqrt(u1u1 / (1.0e-32 + vdotv));
		cont = continuity(r2r2, vdotv, neq, npno);
		++count;
		if(h->verbose)
			fprintf(stderr, "AhatP (%03d) v %12.6e dv/v %9.3e p %12.6e dp/p %9.3e cont %9.3e mg %d\n", count,
			        std::sqrt(vdotv / neq), dvelocity, std::sqrt(pdotp / npno), dpressure, cont, h->stats.mg_passes);
		sh = s1; s1 = s2; s2 = sh;
		sh = r0; r0 = r1; r1 = r2; r2 = sh;
		sh = z0; z0 = z1; z1 = sh;
	}
	h->r0 = r0; h->r1 = r1; h->r2 = r2; h->z0 = z0; h->z1 = z1; h->s1 = s1; h->s2 = s2;
	*steps_max = count;
	if(initial_residual)
		*initial_residual = residual;
	h->stats.uzawa_iterations = count;
	h->stats.initial_residual = residual;
	return CITCOM_GPU_OK;
}

int construct_stiffness(citcom_gpu *h)
{
	const citcom_gpu_config &c = h->cfg;
	const int lmax = h->L - 1;
	for(int l = 0; l < h->L; ++l)
	{
		const bool need64 = (c.precision == CITCOM_GPU_FP64) || l == lmax;
		const bool need32 = (c.precision == CITCOM_GPU_MIXED);
		if(h->geodf[l])
			launch_assemble_df(h->st, h->lv[l], h->geodf[l], h->evi[l], h->eta2[l], c.aug_lagr, need64 ? h->K64[l] : nullptr,
			                   need32 ? h->K32[l] : nullptr, l == lmax ? h->K32lo : nullptr, need64 ? h->BI64[l] : nullptr,
			                   need32 ? h->BI32[l] : nullptr);
		else
			launch_assemble(h->st, h->lv[l], h->geo[l], h->evi[l], c.aug_lagr, c.aug_number, need64 ? h->K64[l] : nullptr,
			                need32 ? h->K32[l] : nullptr, need64 ? h->BI64[l] : nullptr, need32 ? h->BI32[l] : nullptr);
		if(h->Kt32[l])
			launch_tiny_stencil(h->st, h->lv[l], h->K32[l], h->Kt32[l]);
		if(h->eta32[l])
			launch_mf_eta32(h->st, h->lv[l], h->evi[l], h->eta32[l]);
		if(l == 0 && h->co_dense)
			launch_coarse_dense_build(h->st, h->lv[0], h->Kt32[0], h->BI32[0], c.vlowstep, h->co_dense_work, h->co_dense,
			                          h->dscal + S_ERR);
		if(l == 1 && h->co_dense1)
			launch_dense_build_gs(h->st, h->lv[1], h->K32[1], h->BI32[1], h->co_dense1_cycles, h->co_dense1);
	}
	launch_bpi(h->st, h->lv[lmax], h->geo[lmax], h->BI64[lmax], h->BPI, c.precond);
	CK(cudaGetLastError());
	h->stiffness_ready = true;
	return CITCOM_GPU_OK;
}

int project_viscosity(citcom_gpu *h)
{
	for(int l = h->L - 1; l > 0; --l)
		launch_project_viscosity(h->st, h->lv[l], h->lv[l - 1], h->geo[l], h->geo[l - 1], h->evi[l], h->evi[l - 1], h->visc_work[0],
		                         h->visc_work[1]);
	CK(cudaGetLastError());
	h->visc_ready = true;
	return CITCOM_GPU_OK;
}

// get_system_viscosity (Viscosity_structures.c:369-455) on the resident T
// (and, with stress dependence, the resident V), then project_viscosity
int viscosity_from_device_T(citcom_gpu *h)
{
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	const Rheo r = rheo_of(h->cfg);
	launch_visc_from_T(h->st, Lf, h->geo[lmax], r, h->T, h->evi[lmax]);
	if(h->cfg.sdepv)
	{
		// the first call of visc_from_S takes a unit strain rate (:787-790)
		const double *ed = nullptr;
		if(h->sdepv_visits > 0)
		{
			launch_strain_rate(h->st, Lf, h->geo[lmax], h->V, h->edot);
			ed = h->edot;
		}
		launch_visc_from_S(h->st, Lf, h->geo[lmax], r, h->T, ed, h->evi[lmax]);
		h->sdepv_visits++;
	}
	return project_viscosity(h);
}

int forces_from_device_T(citcom_gpu *h)
{
	const int lmax = h->L - 1;
	launch_buoyancy(h->st, h->lv[lmax], h->geo[lmax], h->cfg.rayleigh, h->T, h->buoy);
	launch_forces(h->st, h->lv[lmax], h->geo[lmax], h->buoy, h->F);
	CK(cudaGetLastError());
	return CITCOM_GPU_OK;
}

// general_stokes_solver on the resident T, U, P (Drive_solvers.c:45-165)
int stokes_resident(citcom_gpu *h)
{
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	CK(cudaEventRecord(h->ev0, h->st));
	h->stats.del2_calls = 0;
	h->stats.mg_passes = 0;
	h->stats.smoother_ms = 0.0;
	h->stats.smoother_sweeps = 0;
	h->stats.pass_ms = 0.0;
	launch_strip(h->st, Lf, h->U);  // velocities_conform_bcs with VB = 0
	TRY(forces_from_device_T(h));
	// the viscosity iteration of stress-dependent rheologies (Drive_solvers.c:
	// 120-159): viscosity from T and the last V, operator, solve, damped
	// update, until |dU| / |U| <= sdepv_misfit or max_sdep_visc_iter
	const bool iterate = h->cfg.sdepv != 0;
	const bool update = h->cfg.tdepv || iterate;
	bool asm_timed = false;
	int vcount = 0, uzawa_total = 0;
	double misfit = 0.0;
	do
	{
		if(update || !h->visc_ready)
			TRY(viscosity_from_device_T(h));
		if(update || !h->stiffness_ready)
		{
			CK(cudaEventRecord(h->ev_asm[0], h->st));
			TRY(construct_stiffness(h));
			CK(cudaEventRecord(h->ev_asm[1], h->st));
			asm_timed = true;
		}
		int steps = h->cfg.piterations;
		double r0;
		TRY(uzawa(h, h->U, h->P, h->F, h->cfg.accuracy, &steps, &r0));
		uzawa_total += steps;
		launch_v_from_vector(h->st, Lf, h->U, h->V);
		++vcount;
		if(iterate)
		{
			const double alpha = h->cfg.sdepv_iter_damp;
			if(std::fabs(alpha - 1.0) > 1e-7)
				launch_lin2(h->st, Lf.neq, h->U, alpha, h->U, 1.0 - alpha, h->oldU);
			launch_lin2(h->st, Lf.neq, h->r64, 1.0, h->U, -1.0, h->oldU);  // delta_U
			CK(cudaMemcpyAsync(h->oldU, h->U, sizeof(double) * Lf.neq, cudaMemcpyDeviceToDevice, h->st));
			launch_dots4(h->st, Lf.neq, h->U, h->U, h->r64, h->r64, nullptr, nullptr, nullptr, nullptr, red_of(h),
			             h->dscal + S_DOT);
			TRY(readback(h, S_DOT, 2));
			const double uu = std::sqrt(h->hscal[S_DOT]), dd = std::sqrt(h->hscal[S_DOT + 1]);
			misfit = uu != 0.0 ? dd / uu : dd;
		}
	} while(iterate && misfit > h->cfg.sdepv_misfit && vcount < h->cfg.max_sdep_visc_iter);
	h->stats.uzawa_iterations = uzawa_total;
	h->stats.visc_iterations = vcount;
	h->stats.visc_misfit = misfit;
	CK(cudaMemcpyAsync(h->T_sol, h->T, sizeof(double) * Lf.nno, cudaMemcpyDeviceToDevice, h->st));
	h->T_sol_valid = true;
	CK(cudaEventRecord(h->ev1, h->st));
	CK(cudaEventSynchronize(h->ev1));
	float ms = 0.f;
	CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
	h->stats.stokes_ms = ms;
	h->stats.assembly_ms = 0.0;
	if(asm_timed && cudaEventElapsedTime(&ms, h->ev_asm[0], h->ev_asm[1]) == cudaSuccess)
		h->stats.assembly_ms = ms;
	return CITCOM_GPU_OK;
}

// PG_timestep (Advection_diffusion.c:251-345) on the resident T, Tdot, V
int pg_timestep(citcom_gpu *h, citcom_gpu_advection *adv)
{
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	const Geo *geo = h->geo[lmax];
	const citcom_gpu_config &c = h->cfg;
	cudaStream_t st = h->st;
	const double gamma = 0.5;
	double dt;
	// std_timestep (:737-810)
	if(c.fixed_timestep != 0.0)
		dt = c.fixed_timestep;
	else
	{
		const double diff_ts = h->diff_ts;
		launch_adv_timestep(st, Lf, geo, h->V, red_of(h), h->dscal + S_MIN);
		TRY(readback(h, S_MIN, 1));
		const double adv_ts = c.finetunedt * h->hscal[S_MIN];
		dt = 1.0e-32 + (adv_ts < diff_ts ? adv_ts : diff_ts);
	}
	CK(cudaMemcpyAsync(h->T1, h->T, sizeof(double) * Lf.nno, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(h->Tdot1, h->Tdot, sizeof(double) * Lf.nno, cudaMemcpyDeviceToDevice, st));
	launch_tmax(st, Lf.nno, h->T, red_of(h), h->dscal + S_MAX);
	TRY(readback(h, S_MAX, 1));
	const double T_interior1 = h->hscal[S_MAX];
	double dt_reduced = 1.0, T_interior;
	int sub = 1, iredo;
	do
	{
		dt *= dt_reduced;
		iredo = 0;
		launch_predictor(st, Lf, h->T, h->Tdot, dt, gamma);
		for(int pass = 0; pass < c.adv_sub_iterations; ++pass)
		{
			launch_pg_residual(st, Lf, geo, h->T, h->Tdot, h->V, c.Q0, h->Eres);
			launch_pg_gather(st, Lf, geo, h->Eres, h->DTdot);
			launch_corrector(st, Lf, h->T, h->Tdot, h->DTdot, dt, gamma);
		}
		launch_tmax(st, Lf.nno, h->T, red_of(h), h->dscal + S_MAX);
		TRY(readback(h, S_MAX, 1));
		T_interior = h->hscal[S_MAX];
		if(T_interior / T_interior1 > 1.01)
		{
			CK(cudaMemcpyAsync(h->T, h->T1, sizeof(double) * Lf.nno, cudaMemcpyDeviceToDevice, st));
			CK(cudaMemcpyAsync(h->Tdot, h->Tdot1, sizeof(double) * Lf.nno, cudaMemcpyDeviceToDevice, st));
			iredo = 1;
			dt_reduced *= 0.5;
			++sub;
		}
	} while(iredo == 1 && sub <= 5);
	launch_conform_T(st, Lf, h->T);
	CK(cudaGetLastError());
	if(adv)
	{
		adv->timestep = dt;
		adv->elapsed_time += dt;
		adv->T_interior = T_interior;
		adv->last_sub_iterations = 1;
	}
	return CITCOM_GPU_OK;
}

int check_handle(const citcom_gpu *h) { return h ? CITCOM_GPU_OK : CITCOM_GPU_ERR_ARG; }

int check_level(citcom_gpu *h, int lev)
{
	if(lev < 0 || lev >= h->L)
		return fail(h, CITCOM_GPU_ERR_ARG, "level %d outside 0..%d", lev, h->L - 1);
	return CITCOM_GPU_OK;
}

int h2d(citcom_gpu *h, void *dst, const void *src, size_t bytes)
{
	if(!src)
		return fail(h, CITCOM_GPU_ERR_ARG, "null input pointer");
	CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->st));
	return CITCOM_GPU_OK;
}

int d2h(citcom_gpu *h, void *dst, const void *src, size_t bytes)
{
	if(!dst)
		return CITCOM_GPU_OK;
	CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->st));
	return CITCOM_GPU_OK;
}

int sync(citcom_gpu *h)
{
	CK(cudaStreamSynchronize(h->st));
	CK(cudaGetLastError());
	return CITCOM_GPU_OK;
}

template <typename T> int alloc_mg(citcom_gpu *h, MG<T> &B)
{
	for(int l = 0; l < h->L; ++l)
	{
		const size_t n = h->lv[l].neq + 2;
		TRY(dalloc(h, &B.vel[l], n));
		TRY(dalloc(h, &B.res[l], n));
		TRY(dalloc(h, &B.rhs[l], n));
		TRY(dalloc(h, &B.fl[l], n));
		TRY(dalloc(h, &B.del[l], n));
		TRY(dalloc(h, &B.AU[l], n));
	}
	return CITCOM_GPU_OK;
}

} // namespace

// ====================================================================== C ABI

extern "C" {

// why the last citcom_gpu_create of the process failed (no handle to hold it)
static char g_create_err[256];

static int create_failed(int r, const char *msg)
{
	snprintf(g_create_err, sizeof(g_create_err), "%s", msg);
	return r;
}

int citcom_gpu_create(const citcom_gpu_config *cfg, citcom_gpu **out)
{
	if(!cfg || !out)
		return create_failed(CITCOM_GPU_ERR_ARG, "null argument");
	*out = nullptr;
	if(cfg->levels < 1 || cfg->levels > CITCOM_MAX_LEVELS || cfg->mgunit[0] < 1 || cfg->mgunit[1] < 1 || cfg->mgunit[2] < 1 ||
	   cfg->precision < CITCOM_GPU_FP64 || cfg->precision > CITCOM_GPU_MIXED || cfg->num_mat < 1 || cfg->num_mat > 8)
		return create_failed(CITCOM_GPU_ERR_ARG, "invalid configuration (levels, mgunit, precision or num_mat)");
	int ndev = 0;
	if(cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
	{
		cudaGetLastError();
		return create_failed(CITCOM_GPU_ERR_CUDA, "no usable CUDA device (there is no CPU fallback)");
	}
	citcom_gpu *h = new citcom_gpu();
	memset(h->err, 0, sizeof(h->err));
	h->cfg = *cfg;
	h->L = cfg->levels;
	h->mg_exec = nullptr;
	h->stiffness_ready = false;
	h->visc_ready = false;
	{
		const char *v = getenv("CITCOM_GPU_VERBOSE");
		h->verbose = v && v[0] && v[0] != '0';
		const char *g = getenv("CITCOM_GPU_NO_GRAPH");
		h->no_graph = g && g[0] && g[0] != '0';
		const char *t = getenv("CITCOM_GPU_LEVEL_TIMING");
		h->level_timing = t && t[0] && t[0] != '0';
		if(h->level_timing)
			h->no_graph = true;
		const char *tn = getenv("CITCOM_GPU_NO_TINY");
		h->no_tiny = tn && tn[0] && tn[0] != '0';
		const char *mf = getenv("CITCOM_GPU_MF");
		h->mf = mf && mf[0] && mf[0] != '0';
		const char *fa = getenv("CITCOM_GPU_FP64_ASSEMBLY");
		h->fp64_assembly = fa && fa[0] && fa[0] != '0';
		const char *ns = getenv("CITCOM_GPU_NO_SPLIT");
		h->no_split = ns && ns[0] && ns[0] != '0';
		const char *q = getenv("CITCOM_GPU_NO_PDL");
		if(q && q[0] && q[0] != '0')
			g_use_pdl = 0;
		const char *nc = getenv("CITCOM_GPU_NO_CLUSTER");
		h->co_LC = (nc && nc[0] && nc[0] != '0') ? -2 : -1;
	}
	memset(&h->stats, 0, sizeof(h->stats));
	int r = CITCOM_GPU_OK;
#define TRYC(call)                  \
	do                              \
	{                               \
		r = (call);                 \
		if(r != CITCOM_GPU_OK)      \
			goto failed;            \
	} while(0)
	{
		if(kernels_init() != 0)
		{
			r = fail(h, CITCOM_GPU_ERR_CUDA, "kernel attribute set-up failed");
			goto failed;
		}
		bool ev_ok = true;
		for(int k = 0; k < 8; ++k)
			ev_ok = ev_ok && cudaEventCreate(&h->ev_gs[k]) == cudaSuccess;
		for(int k = 0; k < 2; ++k)
			ev_ok = ev_ok && cudaEventCreate(&h->ev_pass[k]) == cudaSuccess && cudaEventCreate(&h->ev_energy[k]) == cudaSuccess &&
			        cudaEventCreate(&h->ev_asm[k]) == cudaSuccess;
		if(!ev_ok || cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
		   cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
		{
			r = fail(h, CITCOM_GPU_ERR_CUDA, "stream/event creation failed");
			goto failed;
		}
		for(int l = 0; l < h->L; ++l)
			make_level(*cfg, l, h->lv[l]);
		const int lmax = h->L - 1;
		const Lvl &Lf = h->lv[lmax];
		// the coarse levels that the cluster program serves (mixed precision)
		{
			const bool allowed = h->co_LC == -1 && cfg->precision == CITCOM_GPU_MIXED;
			h->co_LC = -1;
			h->co_cluster = 0;
			h->co_smem = 0;
			if(allowed && coarse_init(&h->co_cluster) == 0)
			{
				for(int l = 0; l < lmax && l < CO_MAX_LEV; ++l)
				{
					if(!coarse_level_ok(h->lv[l], l, h->co_cluster, &h->co_local[l]))
						break;
					h->co_LC = l;
					h->co_smem = std::max(h->co_smem, coarse_smem(h->lv[l], h->co_local[l]));
				}
				if(h->co_LC < 1)
					h->co_LC = -1;
			}
			cudaGetLastError();
			h->co_prog.n = 0;
		}
		set_l2_policy(h);
		for(int l = 0; l < h->L; ++l)
		{
			const Lvl &L = h->lv[l];
			{
				std::vector<Geo> g(geo_count(L));
				geo_fill_host(L, g.data());
				TRYC(dalloc(h, &h->geo[l], g.size()));
				if(cudaMemcpy(h->geo[l], g.data(), sizeof(Geo) * g.size(), cudaMemcpyHostToDevice) != cudaSuccess)
				{
					r = fail(h, CITCOM_GPU_ERR_CUDA, "geometry upload failed");
					goto failed;
				}
				h->geodf[l] = nullptr;
				h->eta2[l] = nullptr;
				if(cfg->precision == CITCOM_GPU_MIXED && !h->fp64_assembly)
				{
					// the mixed configuration assembles in double-float: the
					// element kernels of every geometry column as FP32 pairs,
					// word-major (word w of column c at w * ncol + c)
					const size_t ncol = g.size();
					std::vector<float> gt((size_t)GEODF_WORDS * ncol);
					GeoDF one;
					for(size_t cc = 0; cc < ncol; ++cc)
					{
						geo_df_fill(g[cc], cfg->aug_lagr, cfg->aug_number, &one);
						const float *wv = reinterpret_cast<const float *>(&one);
						for(int wd = 0; wd < GEODF_WORDS; ++wd)
							gt[(size_t)wd * ncol + cc] = wv[wd];
					}
					TRYC(dalloc(h, &h->geodf[l], gt.size()));
					TRYC(dalloc(h, &h->eta2[l], (size_t)8 * L.nel));
					if(cudaMemcpy(h->geodf[l], gt.data(), sizeof(float) * gt.size(), cudaMemcpyHostToDevice) != cudaSuccess)
					{
						r = fail(h, CITCOM_GPU_ERR_CUDA, "geometry upload failed");
						goto failed;
					}
				}
				if(l == lmax)
				{
					// std_timestep's diffusive limit: half the smallest squared element size (:760-772)
					h->diff_ts = 1.0e8;
					for(const Geo &e : g)
						for(int d = 0; d < 3; ++d)
							h->diff_ts = std::fmin(h->diff_ts, e.size[d] * e.size[d]);
					h->diff_ts *= 0.5;
				}
			}
			TRYC(dalloc(h, &h->evi[l], (size_t)L.nel * 8));
			const bool need64 = (cfg->precision == CITCOM_GPU_FP64) || l == lmax;
			const bool need32 = (cfg->precision == CITCOM_GPU_MIXED);
			h->K64[l] = nullptr;
			h->BI64[l] = nullptr;
			h->K32[l] = nullptr;
			h->BI32[l] = nullptr;
			h->K32lo = l == lmax ? nullptr : h->K32lo;
			// the finest FP64 operator of the mixed box: the FP32 stencil plus
			// its FP32 remainder, applied in double-float (k_tile_split)
			const bool split = l == lmax && cfg->precision == CITCOM_GPU_MIXED && h->geodf[l] && !L.aos && !h->no_split;
			if(need64)
			{
				if(split)
				{
					TRYC(dalloc(h, &h->K32lo, cg_kwords(L)));
					TRYC(dalloc(h, &h->usplit, (size_t)L.neq));
				}
				else
					TRYC(dalloc(h, &h->K64[l], cg_kwords(L)));
				TRYC(dalloc(h, &h->BI64[l], (size_t)3 * L.npad));
			}
			h->Kt32[l] = nullptr;
			h->eta32[l] = nullptr;
			if(need32)
			{
				TRYC(dalloc(h, &h->K32[l], cg_kwords(L)));
				TRYC(dalloc(h, &h->BI32[l], (size_t)3 * L.npad));
				if(gs_tiny_fits(L, sizeof(float)) || l <= h->co_LC)
					TRYC(dalloc(h, &h->Kt32[l], (size_t)63 * L.nno));
				// box levels smoothed colour by colour (not by the single-CTA or
				// cluster programs): matrix-free unless switched off
				else if(h->mf && !L.aos && !L.sphere && !gs_small_fits(L, sizeof(float)))
					TRYC(dalloc(h, &h->eta32[l], (size_t)8 * L.nel));
			}
			h->mg64.K[l] = h->K64[l];
			h->mg64.BI[l] = h->BI64[l];
			h->mg32.K[l] = h->K32[l];
			h->mg32.BI[l] = h->BI32[l];
		}
		if(cfg->precision == CITCOM_GPU_FP64)
			TRYC(alloc_mg(h, h->mg64));
		else
			TRYC(alloc_mg(h, h->mg32));
		memset(&h->co_lv, 0, sizeof(h->co_lv));
		h->co_lv.nlev = h->co_LC + 1;
		for(int l = 0; l <= h->co_LC; ++l)
		{
			h->co_lv.win[l] = coarse_window(h->lv[l], h->co_cluster);
			h->co_lv.L[l] = h->lv[l];
			h->co_lv.Kt[l] = h->Kt32[l];
			h->co_lv.geo[l] = h->geo[l];
			h->co_lv.BI[l] = h->BI32[l];
			for(int v = 0; v < CO_NVEC; ++v)
				h->co_lv.vec[l][v] = mg_vec(h->mg32, l, v);
		}
		h->co_dense = nullptr;
		h->co_dense_work = nullptr;
		if(h->co_LC >= 0 && h->co_local[0] && h->lv[0].neq <= CO_DENSE_MAX_EQ)
		{
			const char *nd = getenv("CITCOM_GPU_NO_DENSE");
			if(!(nd && nd[0] && nd[0] != '0'))
			{
				const size_t n = (size_t)h->lv[0].neq;
				TRYC(dalloc(h, &h->co_dense, n * n));
				TRYC(dalloc(h, &h->co_dense_work, 2 * n * n));
			}
		}
		h->co_dense1 = nullptr;
		h->co_dense1_cycles = cfg->down_heavy;
		if(h->co_dense && h->co_LC >= 1 && !h->co_local[1] && h->L > 2 && h->lv[1].neq <= CO_DENSE1_MAX_EQ)
		{
			int maxc = 0;
			for(int c = 0; c < 8; ++c)
				maxc = std::max(maxc, h->lv[1].coff[c + 1] - h->lv[1].coff[c]);
			if(maxc <= CO_DENSE1_MAX_COLOUR)
			{
				const size_t n = (size_t)h->lv[1].neq;
				TRYC(dalloc(h, &h->co_dense1, n * n));
			}
		}
		for(int l = 0; l < CO_MAX_LEV; ++l)
			h->co_lv.dense[l] = nullptr;
		h->co_lv.dense[0] = h->co_dense;
		h->co_lv.dense[1] = h->co_dense1;
		TRYC(dalloc(h, &h->BPI, Lf.nel));
		TRYC(dalloc(h, &h->visc_work[0], Lf.nno));
		TRYC(dalloc(h, &h->visc_work[1], Lf.nno));
		TRYC(dalloc(h, &h->U, Lf.neq + 2));
		TRYC(dalloc(h, &h->P, Lf.nel));
		TRYC(dalloc(h, &h->F, Lf.neq + 2));
		TRYC(dalloc(h, &h->T, Lf.nno));
		TRYC(dalloc(h, &h->Tdot, Lf.nno));
		TRYC(dalloc(h, &h->V, (size_t)3 * Lf.nno));
		TRYC(dalloc(h, &h->buoy, Lf.nno + Lf.noz));
		TRYC(dalloc(h, &h->r0, Lf.nel));
		TRYC(dalloc(h, &h->r1, Lf.nel));
		TRYC(dalloc(h, &h->r2, Lf.nel));
		TRYC(dalloc(h, &h->z0, Lf.nel));
		TRYC(dalloc(h, &h->z1, Lf.nel));
		TRYC(dalloc(h, &h->s1, Lf.nel));
		TRYC(dalloc(h, &h->s2, Lf.nel));
		TRYC(dalloc(h, &h->Ah, Lf.neq + 2));
		TRYC(dalloc(h, &h->u1, Lf.neq + 2));
		TRYC(dalloc(h, &h->r64, Lf.neq + 2));
		TRYC(dalloc(h, &h->oldU, Lf.neq + 2));
		TRYC(dalloc(h, &h->T_sol, Lf.nno));
		TRYC(dalloc(h, &h->edot, Lf.nel));
		TRYC(dalloc(h, &h->Eres, (size_t)8 * Lf.nel));
		TRYC(dalloc(h, &h->DTdot, Lf.nno));
		TRYC(dalloc(h, &h->T1, Lf.nno));
		TRYC(dalloc(h, &h->Tdot1, Lf.nno));
		TRYC(dalloc(h, &h->hf_work, Lf.nno + Lf.nel));
		TRYC(dalloc(h, &h->dscal, S_COUNT));
		h->co_lv.err = h->dscal + S_ERR;
		TRYC(dalloc(h, &h->red.partials, (size_t)RED_MAX_BLOCKS * 8));
		TRYC(dalloc(h, &h->red.counter, 1));
		if(cudaMallocHost((void **)&h->hscal, S_COUNT * sizeof(double)) != cudaSuccess)
		{
			r = fail(h, CITCOM_GPU_ERR_CUDA, "pinned scalar buffer");
			goto failed;
		}
		if(cudaDeviceSynchronize() != cudaSuccess)
		{
			r = fail(h, CITCOM_GPU_ERR_CUDA, "initialisation failed");
			goto failed;
		}
	}
#undef TRYC
	*out = h;
	return CITCOM_GPU_OK;
failed:
	create_failed(r, h->err);
	citcom_gpu_destroy(h);
	return r;
}

void citcom_gpu_destroy(citcom_gpu *h)
{
	if(!h)
		return;
	if(h->warm)
		h->warm->h = nullptr;
	if(h->level_timing)
		for(int l = 0; l < h->L; ++l)
			fprintf(stderr, "level %d (%d nodes, %s): %ld smoother calls, %ld sweeps, %.3f ms total, %.2f us/call, %.2f us/sweep\n",
			        l, h->lv[l].nno, h->cfg.precision == CITCOM_GPU_FP64 ? "fp64" : "fp32", h->lt_calls[l], h->lt_sweeps[l],
			        h->lt_ms[l], h->lt_calls[l] ? 1e3 * h->lt_ms[l] / h->lt_calls[l] : 0.0,
			        h->lt_sweeps[l] ? 1e3 * h->lt_ms[l] / h->lt_sweeps[l] : 0.0);
	if(h->st)
		cudaStreamSynchronize(h->st);
	if(h->st_out)
	{
		cudaStreamSynchronize(h->st_out);
		cudaStreamDestroy(h->st_out);
	}
	if(h->ev_snap)
		cudaEventDestroy(h->ev_snap);
	if(h->ev_out)
		cudaEventDestroy(h->ev_out);
	if(h->mg_exec)
		cudaGraphExecDestroy(h->mg_exec);
	for(void *p : h->allocs)
		cudaFree(p);
	if(h->hscal)
		cudaFreeHost(h->hscal);
	if(h->ev0)
		cudaEventDestroy(h->ev0);
	if(h->ev1)
		cudaEventDestroy(h->ev1);
	for(int k = 0; k < 8; ++k)
		if(h->ev_gs[k])
			cudaEventDestroy(h->ev_gs[k]);
	for(int k = 0; k < 2; ++k)
	{
		if(h->ev_pass[k])
			cudaEventDestroy(h->ev_pass[k]);
		if(h->ev_energy[k])
			cudaEventDestroy(h->ev_energy[k]);
		if(h->ev_asm[k])
			cudaEventDestroy(h->ev_asm[k]);
	}
	if(h->st)
		cudaStreamDestroy(h->st);
	delete h;
}

const char *citcom_gpu_error_string(const citcom_gpu *h)
{
	if(h)
		return h->err;
	return g_create_err[0] ? g_create_err : "null handle";
}

int citcom_gpu_level_dims(const citcom_gpu *h, int lev, int dims[6])
{
	if(!h || !dims || lev < 0 || lev >= h->L)
		return CITCOM_GPU_ERR_ARG;
	const Lvl &L = h->lv[lev];
	dims[0] = L.nox;
	dims[1] = L.noy;
	dims[2] = L.noz;
	dims[3] = L.nno;
	dims[4] = L.nel;
	dims[5] = L.neq;
	return CITCOM_GPU_OK;
}

int citcom_gpu_get_system_viscosity(citcom_gpu *h, const double *T)
{
	TRY(check_handle(h));
	const Lvl &Lf = h->lv[h->L - 1];
	TRY(h2d(h, h->T, T, sizeof(double) * Lf.nno));
	TRY(viscosity_from_device_T(h));
	return sync(h);
}

int citcom_gpu_set_viscosity(citcom_gpu *h, int lev, const double *evi)
{
	TRY(check_handle(h));
	TRY(check_level(h, lev));
	TRY(h2d(h, h->evi[lev], evi, sizeof(double) * 8 * h->lv[lev].nel));
	h->visc_ready = true;
	return sync(h);
}

int citcom_gpu_get_viscosity(citcom_gpu *h, int lev, double *evi)
{
	TRY(check_handle(h));
	TRY(check_level(h, lev));
	TRY(d2h(h, evi, h->evi[lev], sizeof(double) * 8 * h->lv[lev].nel));
	return sync(h);
}

int citcom_gpu_construct_stiffness_B_matrix(citcom_gpu *h)
{
	TRY(check_handle(h));
	TRY(construct_stiffness(h));
	return sync(h);
}

int citcom_gpu_assemble_forces(citcom_gpu *h, const double *T, double *F, double *buoyancy)
{
	TRY(check_handle(h));
	const Lvl &Lf = h->lv[h->L - 1];
	TRY(h2d(h, h->T, T, sizeof(double) * Lf.nno));
	TRY(forces_from_device_T(h));
	TRY(d2h(h, F, h->F, sizeof(double) * Lf.neq));
	TRY(d2h(h, buoyancy, h->buoy, sizeof(double) * Lf.nno));
	return sync(h);
}

int citcom_gpu_solve_Ahat_p_fhat_device(citcom_gpu *h, double *dV, double *dP, const double *dF, double imp, int *steps_max,
                                        double *initial_residual)
{
	TRY(check_handle(h));
	if(!dV || !dP || !dF || !steps_max)
		return fail(h, CITCOM_GPU_ERR_ARG, "null argument");
	h->stats.del2_calls = 0;
	h->stats.mg_passes = 0;
	h->stats.smoother_ms = 0.0;
	h->stats.smoother_sweeps = 0;
	h->stats.pass_ms = 0.0;
	CK(cudaEventRecord(h->ev0, h->st));
	TRY(uzawa(h, dV, dP, dF, imp, steps_max, initial_residual));
	CK(cudaEventRecord(h->ev1, h->st));
	TRY(sync(h));
	float ms = 0.f;
	CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
	h->stats.stokes_ms = ms;
	return CITCOM_GPU_OK;
}

int citcom_gpu_solve_Ahat_p_fhat(citcom_gpu *h, double *V, double *P, const double *F, double imp, int *steps_max,
                                 double *initial_residual)
{
	TRY(check_handle(h));
	const Lvl &Lf = h->lv[h->L - 1];
	TRY(h2d(h, h->U, V, sizeof(double) * Lf.neq));
	TRY(h2d(h, h->P, P, sizeof(double) * Lf.nel));
	TRY(h2d(h, h->F, F, sizeof(double) * Lf.neq));
	TRY(citcom_gpu_solve_Ahat_p_fhat_device(h, h->U, h->P, h->F, imp, steps_max, initial_residual));
	TRY(d2h(h, V, h->U, sizeof(double) * Lf.neq));
	TRY(d2h(h, P, h->P, sizeof(double) * Lf.nel));
	return sync(h);
}

int citcom_gpu_solve_constrained_flow_iterative(citcom_gpu *h, double *U, double *P, const double *F, double *V)
{
	TRY(check_handle(h));
	const Lvl &Lf = h->lv[h->L - 1];
	int steps = h->cfg.piterations;
	double r0;
	TRY(h2d(h, h->U, U, sizeof(double) * Lf.neq));
	TRY(h2d(h, h->P, P, sizeof(double) * Lf.nel));
	TRY(h2d(h, h->F, F, sizeof(double) * Lf.neq));
	TRY(citcom_gpu_solve_Ahat_p_fhat_device(h, h->U, h->P, h->F, h->cfg.accuracy, &steps, &r0));
	launch_v_from_vector(h->st, Lf, h->U, h->V);
	TRY(d2h(h, U, h->U, sizeof(double) * Lf.neq));
	TRY(d2h(h, P, h->P, sizeof(double) * Lf.nel));
	TRY(d2h(h, V, h->V, sizeof(double) * 3 * Lf.nno));
	return sync(h);
}

int citcom_gpu_general_stokes_solver(citcom_gpu *h, const double *T, double *U, double *P, double *V)
{
	TRY(check_handle(h));
	const Lvl &Lf = h->lv[h->L - 1];
	TRY(h2d(h, h->T, T, sizeof(double) * Lf.nno));
	TRY(h2d(h, h->U, U, sizeof(double) * Lf.neq));
	TRY(h2d(h, h->P, P, sizeof(double) * Lf.nel));
	TRY(stokes_resident(h));
	TRY(d2h(h, U, h->U, sizeof(double) * Lf.neq));
	TRY(d2h(h, P, h->P, sizeof(double) * Lf.nel));
	TRY(d2h(h, V, h->V, sizeof(double) * 3 * Lf.nno));
	return sync(h);
}

int citcom_gpu_PG_timestep(citcom_gpu *h, double *T, double *Tdot, const double *V, citcom_gpu_advection *adv)
{
	TRY(check_handle(h));
	const Lvl &Lf = h->lv[h->L - 1];
	TRY(h2d(h, h->T, T, sizeof(double) * Lf.nno));
	TRY(h2d(h, h->Tdot, Tdot, sizeof(double) * Lf.nno));
	TRY(h2d(h, h->V, V, sizeof(double) * 3 * Lf.nno));
	TRY(pg_timestep(h, adv));
	TRY(d2h(h, T, h->T, sizeof(double) * Lf.nno));
	TRY(d2h(h, Tdot, h->Tdot, sizeof(double) * Lf.nno));
	return sync(h);
}

int citcom_gpu_heat_flux(citcom_gpu *h, const double *T, const double *V, double *nut, double *nub)
{
	TRY(check_handle(h));
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	const double *dT = h->T, *dV = h->V;
	if(T)
		TRY(h2d(h, h->T, T, sizeof(double) * Lf.nno));
	if(V)
		TRY(h2d(h, h->V, V, sizeof(double) * 3 * Lf.nno));
	launch_heat_flux(h->st, Lf, h->geo[lmax], dT, dV, h->hf_work, red_of(h), h->dscal + S_NU);
	TRY(readback(h, S_NU, 4));
	// Nu = sum of (4-node flux sum x element volume) / (4 x sum of volumes) (Process_buoyancy.c:163-196)
	if(nut)
		*nut = h->hscal[S_NU] / (4.0 * h->hscal[S_NU + 2]);
	if(nub)
		*nub = h->hscal[S_NU + 1] / (4.0 * h->hscal[S_NU + 3]);
	return CITCOM_GPU_OK;
}

int citcom_gpu_vrms(citcom_gpu *h, const double *V, double *vrms)
{
	TRY(check_handle(h));
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	if(V)
		TRY(h2d(h, h->V, V, sizeof(double) * 3 * Lf.nno));
	launch_vrms(h->st, Lf, h->geo[lmax], h->V, red_of(h), h->dscal + S_VRMS);
	TRY(readback(h, S_VRMS, 2));
	if(vrms)
		*vrms = std::sqrt(h->hscal[S_VRMS] / h->hscal[S_VRMS + 1]);
	return CITCOM_GPU_OK;
}

int citcom_gpu_load_state(citcom_gpu *h, const double *T, const double *Tdot, const double *U, const double *P)
{
	TRY(check_handle(h));
	const Lvl &Lf = h->lv[h->L - 1];
	if(T)
		TRY(h2d(h, h->T, T, sizeof(double) * Lf.nno));
	if(Tdot)
		TRY(h2d(h, h->Tdot, Tdot, sizeof(double) * Lf.nno));
	if(U)
		TRY(h2d(h, h->U, U, sizeof(double) * Lf.neq));
	if(P)
		TRY(h2d(h, h->P, P, sizeof(double) * Lf.nel));
	h->state_gen++;
	h->T_sol_valid = false;
	return sync(h);
}

int citcom_gpu_store_state(citcom_gpu *h, double *T, double *Tdot, double *U, double *P, double *V)
{
	TRY(check_handle(h));
	const Lvl &Lf = h->lv[h->L - 1];
	TRY(d2h(h, T, h->T, sizeof(double) * Lf.nno));
	TRY(d2h(h, Tdot, h->Tdot, sizeof(double) * Lf.nno));
	TRY(d2h(h, U, h->U, sizeof(double) * Lf.neq));
	TRY(d2h(h, P, h->P, sizeof(double) * Lf.nel));
	TRY(d2h(h, V, h->V, sizeof(double) * 3 * Lf.nno));
	return sync(h);
}

int citcom_gpu_stokes_resident(citcom_gpu *h)
{
	TRY(check_handle(h));
	TRY(stokes_resident(h));
	return sync(h);
}

int citcom_gpu_step_resident(citcom_gpu *h, citcom_gpu_advection *adv)
{
	TRY(check_handle(h));
	// events of their own: the multigrid graph re-records the smoother and pass
	// events during the solve that follows
	cudaEvent_t a = h->ev_energy[0], b = h->ev_energy[1];
	CK(cudaEventRecord(a, h->st));
	TRY(pg_timestep(h, adv));
	CK(cudaEventRecord(b, h->st));
	TRY(stokes_resident(h));
	TRY(sync(h));
	float ms = 0.f;
	CK(cudaEventElapsedTime(&ms, a, b));
	h->stats.energy_ms = ms;
	return CITCOM_GPU_OK;
}

int citcom_gpu_output_async(citcom_gpu *h, const citcom_gpu_output *o)
{
	TRY(check_handle(h));
	if(!o)
		return fail(h, CITCOM_GPU_ERR_ARG, "null output descriptor");
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	const size_t nno = Lf.nno, nel = Lf.nel, noz = Lf.noz, nsf = (size_t)Lf.nox * Lf.noy;
	// created on first use, each on its own so that a failed call leaves
	// nothing half made
	if(!h->st_out && cudaStreamCreateWithFlags(&h->st_out, cudaStreamNonBlocking) != cudaSuccess)
	{
		h->st_out = nullptr;
		return fail(h, CITCOM_GPU_ERR_CUDA, "output stream creation failed");
	}
	if(!h->ev_snap && cudaEventCreateWithFlags(&h->ev_snap, cudaEventDisableTiming) != cudaSuccess)
	{
		h->ev_snap = nullptr;
		return fail(h, CITCOM_GPU_ERR_CUDA, "output event creation failed");
	}
	if(!h->ev_out && cudaEventCreateWithFlags(&h->ev_out, cudaEventDisableTiming) != cudaSuccess)
	{
		h->ev_out = nullptr;
		return fail(h, CITCOM_GPU_ERR_CUDA, "output event creation failed");
	}
	if(!h->snap)
		TRY(dalloc(h, &h->snap, 8 * nno + 4 * nel + 6 * noz + 2 * nsf + 9));
	double *sT = h->snap, *sV = sT + nno, *sP = sV + 3 * nno, *f = sP + nel, *scratch = f + 3 * nno, *ue = scratch + nno;
	double *H = ue + 3 * nel, *surf = H + 6 * noz, *sums = surf + 2 * nsf, *scal = sums + 6;
	// the staging must not change under a host copy still in flight
	if(h->snap_pending)
		CK(cudaStreamWaitEvent(h->st, h->ev_out, 0));
	if(o->T)
		CK(cudaMemcpyAsync(sT, h->T, sizeof(double) * nno, cudaMemcpyDeviceToDevice, h->st));
	if(o->V)
		CK(cudaMemcpyAsync(sV, h->V, sizeof(double) * 3 * nno, cudaMemcpyDeviceToDevice, h->st));
	if(o->P)
		CK(cudaMemcpyAsync(sP, h->P, sizeof(double) * nel, cudaMemcpyDeviceToDevice, h->st));
	if(o->heatflux || o->heatflux_adv || o->Have || o->surf || o->scalars)
		launch_output_fields(h->st, Lf, h->geo[lmax], h->T, h->V, h->evi[lmax], red_of(h), f, scratch, ue, H, surf, sums, scal);
	CK(cudaEventRecord(h->ev_snap, h->st));
	CK(cudaStreamWaitEvent(h->st_out, h->ev_snap, 0));
	struct
	{
		double *dst;
		const double *src;
		size_t n;
	} cp[8] = {{o->T, sT, nno},           {o->V, sV, 3 * nno},         {o->P, sP, nel},   {o->heatflux, f + 2 * nno, nno},
	           {o->heatflux_adv, f + nno, nno}, {o->Have, H, 6 * noz}, {o->surf, surf, 2 * nsf}, {o->scalars, scal, 3}};
	for(int i = 0; i < 8; ++i)
		if(cp[i].dst)
			CK(cudaMemcpyAsync(cp[i].dst, cp[i].src, sizeof(double) * cp[i].n, cudaMemcpyDeviceToHost, h->st_out));
	CK(cudaEventRecord(h->ev_out, h->st_out));
	h->snap_pending = true;
	return CITCOM_GPU_OK;
}

int citcom_gpu_output_wait(citcom_gpu *h)
{
	TRY(check_handle(h));
	if(h->snap_pending)
		CK(cudaEventSynchronize(h->ev_out));
	h->snap_pending = false;
	return CITCOM_GPU_OK;
}

static int stokes_residuals_impl(citcom_gpu *h, double out[2])
{
	TRY(check_handle(h));
	if(!out)
		return fail(h, CITCOM_GPU_ERR_ARG, "null argument");
	if(!h->stiffness_ready)
		return fail(h, CITCOM_GPU_ERR_STATE, "construct_stiffness_B_matrix has not been called");
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	// momentum: F - K U - G P, with the FP64 operator
	launch_grad(h->st, Lf, h->geo[lmax], h->P, h->Ah);
	fine_kmul64(h, h->U, h->u1);
	launch_sub3(h->st, Lf.neq, h->r64, h->F, h->Ah, h->u1);
	launch_div(h->st, Lf, h->geo[lmax], h->U, h->Eres);
	launch_dots4(h->st, Lf.neq, h->r64, h->r64, h->F, h->F, h->U, h->U, nullptr, nullptr, red_of(h), h->dscal + S_DOT);
	launch_dot(h->st, Lf.nel, h->Eres, h->Eres, red_of(h), h->dscal + S_DOT + 4);
	TRY(readback(h, S_DOT, 5));
	const double rr = h->hscal[S_DOT], ff = h->hscal[S_DOT + 1], uu = h->hscal[S_DOT + 2], dd = h->hscal[S_DOT + 4];
	out[0] = std::sqrt(rr / (ff > 0.0 ? ff : 1.0));
	out[1] = std::sqrt(dd) / (std::sqrt(uu) * std::sqrt((double)Lf.nel / (double)Lf.neq) + 1e-300);
	return CITCOM_GPU_OK;
}

int citcom_gpu_stokes_residuals(citcom_gpu *h, double out[2])
{
	TRY(check_handle(h));
	TRY(device_errors_reset(h));
	TRY(stokes_residuals_impl(h, out));
	return device_errors_check(h, "stokes_residuals");
}

int citcom_gpu_test_hold_tile_copy(void)
{
	return tile_hold_next_copy() == 0 ? CITCOM_GPU_OK : CITCOM_GPU_ERR_CUDA;
}

int citcom_gpu_last_stats(const citcom_gpu *h, citcom_gpu_stats *s)
{
	if(!h || !s)
		return CITCOM_GPU_ERR_ARG;
	*s = h->stats;
	s->kernel_launches = g_kernel_launches;
	return CITCOM_GPU_OK;
}

// ------------------------------------------------------------ single operators

static int op_kmul_impl(citcom_gpu *h, int lev, const double *u, double *Au)
{
	TRY(check_handle(h));
	TRY(check_level(h, lev));
	if(!h->stiffness_ready)
		return fail(h, CITCOM_GPU_ERR_STATE, "construct_stiffness_B_matrix has not been called");
	const Lvl &L = h->lv[lev];
	double *du, *dA;
	if(h->cfg.precision == CITCOM_GPU_FP64 || lev == h->L - 1)
	{
		du = h->cfg.precision == CITCOM_GPU_FP64 ? h->mg64.del[lev] : h->r64;
		dA = h->cfg.precision == CITCOM_GPU_FP64 ? h->mg64.AU[lev] : h->Ah;
		TRY(h2d(h, du, u, sizeof(double) * L.neq));
		if(lev == h->L - 1)
			fine_kmul64(h, du, dA);
		else
			launch_kmul<double>(h->st, L, h->K64[lev], du, dA);
		TRY(d2h(h, Au, dA, sizeof(double) * L.neq));
		return sync(h);
	}
	// FP32 stencil of a coarse level in mixed mode
	std::vector<float> uf(L.neq), af(L.neq);
	for(int i = 0; i < L.neq; ++i)
		uf[i] = (float)u[i];
	TRY(h2d(h, h->mg32.del[lev], uf.data(), sizeof(float) * L.neq));
	launch_kmul<float>(h->st, L, h->K32[lev], h->mg32.del[lev], h->mg32.AU[lev]);
	TRY(d2h(h, af.data(), h->mg32.AU[lev], sizeof(float) * L.neq));
	TRY(sync(h));
	for(int i = 0; i < L.neq; ++i)
		Au[i] = af[i];
	return CITCOM_GPU_OK;
}

int citcom_gpu_op_kmul(citcom_gpu *h, int lev, const double *u, double *Au)
{
	TRY(check_handle(h));
	TRY(device_errors_reset(h));
	TRY(op_kmul_impl(h, lev, u, Au));
	return device_errors_check(h, "op_kmul");
}

static int op_gauss_seidel_impl(citcom_gpu *h, int lev, double *d0, const double *F, double *Ad, int cycles, int guess)
{
	TRY(check_handle(h));
	TRY(check_level(h, lev));
	if(!h->stiffness_ready)
		return fail(h, CITCOM_GPU_ERR_STATE, "construct_stiffness_B_matrix has not been called");
	const Lvl &L = h->lv[lev];
	if(h->cfg.precision != CITCOM_GPU_FP64)
	{
		// mixed configuration: the FP32 smoother of a multigrid level
		if(lev == h->L - 1)
			return fail(h, CITCOM_GPU_ERR_ARG, "the finest level is smoothed in FP32 only inside multi_grid; use a coarser level");
		MG<float> &B = h->mg32;
		std::vector<float> f(L.neq), v(L.neq);
		for(int i = 0; i < L.neq; ++i)
		{
			f[i] = (float)F[i];
			v[i] = guess ? (float)d0[i] : 0.f;
		}
		TRY(h2d(h, B.rhs[lev], f.data(), sizeof(float) * L.neq));
		TRY(h2d(h, B.vel[lev], v.data(), sizeof(float) * L.neq));
		mg_gs<float>(h, B, lev, CO_VEL, CO_RHS, cycles, !guess);
		co_flush(h);
		launch_kmul<float>(h->st, L, B.K[lev], B.vel[lev], B.AU[lev]);
		TRY(d2h(h, v.data(), B.vel[lev], sizeof(float) * L.neq));
		TRY(d2h(h, f.data(), B.AU[lev], sizeof(float) * L.neq));
		TRY(sync(h));
		for(int i = 0; i < L.neq; ++i)
		{
			d0[i] = v[i];
			Ad[i] = f[i];
		}
		return CITCOM_GPU_OK;
	}
	MG<double> &B = h->mg64;
	TRY(h2d(h, B.rhs[lev], F, sizeof(double) * L.neq));
	if(guess)
		TRY(h2d(h, B.vel[lev], d0, sizeof(double) * L.neq));
	gs<double>(h, B, lev, B.vel[lev], B.rhs[lev], cycles, !guess);
	launch_kmul<double>(h->st, L, B.K[lev], B.vel[lev], B.AU[lev]);
	TRY(d2h(h, d0, B.vel[lev], sizeof(double) * L.neq));
	TRY(d2h(h, Ad, B.AU[lev], sizeof(double) * L.neq));
	return sync(h);
}

int citcom_gpu_op_gauss_seidel(citcom_gpu *h, int lev, double *d0, const double *F, double *Ad, int cycles, int guess)
{
	TRY(check_handle(h));
	TRY(device_errors_reset(h));
	TRY(op_gauss_seidel_impl(h, lev, d0, F, Ad, cycles, guess));
	return device_errors_check(h, "op_gauss_seidel");
}

int citcom_gpu_op_project(citcom_gpu *h, int fine_lev, const double *AU, double *AD)
{
	TRY(check_handle(h));
	TRY(check_level(h, fine_lev));
	if(fine_lev < 1)
		return fail(h, CITCOM_GPU_ERR_ARG, "no level below %d", fine_lev);
	const Lvl &Lf = h->lv[fine_lev], &Lc = h->lv[fine_lev - 1];
	double *src, *dst;
	if(h->cfg.precision == CITCOM_GPU_FP64)
	{
		src = h->mg64.del[fine_lev];
		dst = h->mg64.AU[fine_lev - 1];
	}
	else
	{
		src = h->r64;
		dst = h->Ah;
	}
	TRY(h2d(h, src, AU, sizeof(double) * Lf.neq));
	launch_project<double>(h->st, Lf, Lc, h->geo[fine_lev - 1], src, dst);
	TRY(d2h(h, AD, dst, sizeof(double) * Lc.neq));
	return sync(h);
}

int citcom_gpu_op_interp(citcom_gpu *h, int coarse_lev, const double *AD, double *AU)
{
	TRY(check_handle(h));
	TRY(check_level(h, coarse_lev));
	if(coarse_lev >= h->L - 1)
		return fail(h, CITCOM_GPU_ERR_ARG, "no level above %d", coarse_lev);
	const Lvl &Lc = h->lv[coarse_lev], &Lf = h->lv[coarse_lev + 1];
	double *src, *dst;
	if(h->cfg.precision == CITCOM_GPU_FP64)
	{
		src = h->mg64.del[coarse_lev];
		dst = h->mg64.AU[coarse_lev + 1];
	}
	else
	{
		src = h->r64;
		dst = h->Ah;
	}
	TRY(h2d(h, src, AD, sizeof(double) * Lc.neq));
	launch_interp<double>(h->st, Lc, Lf, h->geo[coarse_lev + 1], src, dst);
	TRY(d2h(h, AU, dst, sizeof(double) * Lf.neq));
	return sync(h);
}

int citcom_gpu_op_div(citcom_gpu *h, int lev, const double *U, double *divU)
{
	TRY(check_handle(h));
	TRY(check_level(h, lev));
	const Lvl &L = h->lv[lev];
	TRY(h2d(h, h->r64, U, sizeof(double) * L.neq));
	launch_div(h->st, L, h->geo[lev], h->r64, h->Eres);
	TRY(d2h(h, divU, h->Eres, sizeof(double) * L.nel));
	return sync(h);
}

int citcom_gpu_op_grad(citcom_gpu *h, int lev, const double *P, double *gradP)
{
	TRY(check_handle(h));
	TRY(check_level(h, lev));
	const Lvl &L = h->lv[lev];
	TRY(h2d(h, h->Eres, P, sizeof(double) * L.nel));
	launch_grad(h->st, L, h->geo[lev], h->Eres, h->r64);
	TRY(d2h(h, gradP, h->r64, sizeof(double) * L.neq));
	return sync(h);
}

static int op_multi_grid_impl(citcom_gpu *h, double *d1, double *F, double *residual)
{
	TRY(check_handle(h));
	if(!h->stiffness_ready)
		return fail(h, CITCOM_GPU_ERR_STATE, "construct_stiffness_B_matrix has not been called");
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax];
	if(h->cfg.precision != CITCOM_GPU_FP64)
	{
		// mixed configuration: one FP32 pass (F rounded to float)
		MG<float> &B = h->mg32;
		TRY(h2d(h, h->r64, F, sizeof(double) * Lf.neq));
		launch_copy_d2f(h->st, Lf.neq, B.fl[lmax], h->r64);
		const int pairs = h->n_gs_pairs;
		h->n_gs_pairs = 4;
		mg_pass<float>(h, B);
		h->n_gs_pairs = pairs;
		std::vector<float> v(Lf.neq), r(Lf.neq);
		TRY(d2h(h, v.data(), B.vel[lmax], sizeof(float) * Lf.neq));
		TRY(d2h(h, r.data(), B.res[lmax], sizeof(float) * Lf.neq));
		TRY(sync(h));
		double rr = 0.0;
		for(int i = 0; i < Lf.neq; ++i)
		{
			d1[i] = v[i];
			F[i] = r[i];
			rr += (double)r[i] * r[i];
		}
		if(residual)
			*residual = std::sqrt(rr / Lf.neq);
		return CITCOM_GPU_OK;
	}
	TRY(h2d(h, h->mg64.fl[lmax], F, sizeof(double) * Lf.neq));
	const int pairs = h->n_gs_pairs;
	h->n_gs_pairs = 4;  // no smoother timing outside the captured pass
	mg_pass<double>(h, h->mg64);
	h->n_gs_pairs = pairs;
	launch_dot(h->st, Lf.neq, h->mg64.res[lmax], h->mg64.res[lmax], red_of(h), h->dscal + S_RES);
	TRY(d2h(h, d1, h->mg64.vel[lmax], sizeof(double) * Lf.neq));
	TRY(d2h(h, F, h->mg64.res[lmax], sizeof(double) * Lf.neq));
	TRY(readback(h, S_RES, 1));
	if(residual)
		*residual = std::sqrt(h->hscal[S_RES] / Lf.neq);
	return sync(h);
}

int citcom_gpu_op_multi_grid(citcom_gpu *h, double *d1, double *F, double *residual)
{
	TRY(check_handle(h));
	TRY(device_errors_reset(h));
	TRY(op_multi_grid_impl(h, d1, F, residual));
	return device_errors_check(h, "op_multi_grid");
}

static int op_solve_del2_u_impl(citcom_gpu *h, double *d0, const double *F, double acc, int *valid)
{
	TRY(check_handle(h));
	if(!h->stiffness_ready)
		return fail(h, CITCOM_GPU_ERR_STATE, "construct_stiffness_B_matrix has not been called");
	const Lvl &Lf = h->lv[h->L - 1];
	int v = 0;
	TRY(h2d(h, h->Ah, F, sizeof(double) * Lf.neq));
	h->stats.mg_passes = 0;
	h->stats.del2_calls = 0;
	TRY(solve_del2_u(h, acc, &v));
	TRY(d2h(h, d0, h->u1, sizeof(double) * Lf.neq));
	if(valid)
		*valid = v;
	return sync(h);
}

int citcom_gpu_op_solve_del2_u(citcom_gpu *h, double *d0, const double *F, double acc, int *valid)
{
	TRY(check_handle(h));
	TRY(device_errors_reset(h));
	TRY(op_solve_del2_u_impl(h, d0, F, acc, valid));
	return device_errors_check(h, "op_solve_del2_u");
}

int citcom_gpu_op_diagonals(citcom_gpu *h, int lev, double *BI, double *BPI)
{
	TRY(check_handle(h));
	TRY(check_level(h, lev));
	if(!h->stiffness_ready)
		return fail(h, CITCOM_GPU_ERR_STATE, "construct_stiffness_B_matrix has not been called");
	const Lvl &L = h->lv[lev];
	if(BI)
	{
		std::vector<double> bi(3 * (size_t)L.npad);
		std::vector<float> bf;
		if(h->BI64[lev])
			TRY(d2h(h, bi.data(), h->BI64[lev], sizeof(double) * 3 * L.npad));
		else
		{
			bf.resize(3 * (size_t)L.npad);
			TRY(d2h(h, bf.data(), h->BI32[lev], sizeof(float) * 3 * L.npad));
		}
		TRY(sync(h));
		for(int y = 0; y < L.noy; ++y)
			for(int x = 0; x < L.nox; ++x)
				for(int z = 0; z < L.noz; ++z)
				{
					const int n = cg_node(L, x, y, z), p = cg_pos(L, x, y, z);
					for(int d = 0; d < 3; ++d)
						BI[3 * n + d] = h->BI64[lev] ? bi[3 * (size_t)p + d] : (double)bf[3 * (size_t)p + d];
				}
	}
	if(BPI)
	{
		if(lev != h->L - 1)
			return fail(h, CITCOM_GPU_ERR_ARG, "BPI is kept for the finest level only");
		TRY(d2h(h, BPI, h->BPI, sizeof(double) * L.nel));
	}
	return sync(h);
}

} // extern "C"

// ================================================================ warm start

namespace {

int nn_fail(citcom_nn *n, int code, const char *fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(n->err, sizeof(n->err), fmt, ap);
	va_end(ap);
	return code;
}

// the network's guess of U (finest level) and P from the resident T and viscosity
int nn_guess(citcom_nn *n)
{
	citcom_gpu *h = n->h;
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax], &Lc = h->lv[n->lev];
	launch_nn_inputs(h->st, Lf, Lc, n->r, h->T, h->evi[n->lev], n->x, n->work);
	if(nn_forward(n->net, n->x, n->y) != 0)
		return fail(h, CITCOM_GPU_ERR_CUDA, "warm-start network: forward launch failed");
	launch_nn_guess(h->st, Lf, Lc, n->r, n->y, n->su, n->sp, n->mp, n->work, n->Uv[n->lev], n->Pg);
	for(int l = n->lev; l < lmax; ++l)
	{
		double *dst = (l + 1 == lmax) ? n->Ug : n->Uv[l + 1];
		launch_interp<double>(h->st, h->lv[l], h->lv[l + 1], h->geo[l + 1], n->Uv[l], dst);
		launch_strip(h->st, h->lv[l + 1], dst);
	}
	CK(cudaGetLastError());
	return CITCOM_GPU_OK;
}

// Increment mode: the network maps the temperature change since the last
// solve (T - T_sol) and the viscosity to the change of U and P; the guess is
// Ug = V + dU (stripped), Pg = P + dP.
int nn_increment_guess(citcom_nn *n, const double *V, const double *P)
{
	citcom_gpu *h = n->h;
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax], &Lc = h->lv[n->lev];
	cudaStream_t st = h->st;
	launch_lin2(st, Lf.nno, n->dT, 1.0, h->T, -1.0, h->T_sol);
	launch_nn_inputs(st, Lf, Lc, n->r, n->dT, h->evi[n->lev], n->x, n->work);
	if(nn_forward(n->net, n->x, n->y) != 0)
		return fail(h, CITCOM_GPU_ERR_CUDA, "warm-start network: forward launch failed");
	launch_nn_guess(st, Lf, Lc, n->r, n->y, n->su, n->sp, 0.0, n->work, n->Uv[n->lev], n->Pg);
	for(int l = n->lev; l < lmax; ++l)
	{
		double *dst = (l + 1 == lmax) ? n->Ug : n->Uv[l + 1];
		launch_interp<double>(st, h->lv[l], h->lv[l + 1], h->geo[l + 1], n->Uv[l], dst);
		launch_strip(st, h->lv[l + 1], dst);
	}
	launch_axpby(st, Lf.neq, n->Ug, 1.0, V, 1.0);
	launch_axpby(st, Lf.nel, n->Pg, 1.0, P, 1.0);
	CK(cudaGetLastError());
	return CITCOM_GPU_OK;
}

template <typename T> int nn_alloc(citcom_nn *n, T **p, size_t count)
{
	void *q = nullptr;
	if(cudaMalloc(&q, (count ? count : 1) * sizeof(T)) != cudaSuccess)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "cudaMalloc of %zu bytes failed", count * sizeof(T));
	cudaMemset(q, 0, (count ? count : 1) * sizeof(T));
	n->allocs.push_back(q);
	*p = (T *)q;
	return CITCOM_GPU_OK;
}

int nn_check(citcom_nn *n)
{
	if(!n)
		return CITCOM_GPU_ERR_ARG;
	if(!n->h)
		return nn_fail(n, CITCOM_GPU_ERR_STATE, "the solver of this network was destroyed");
	return CITCOM_GPU_OK;
}

#define NTRY(call)               \
	do                           \
	{                            \
		int r_ = (call);         \
		if(r_ != CITCOM_GPU_OK)  \
			return r_;           \
	} while(0)

// host (V x 2 FP32) -> device network input (V x 16 BF16)
int nn_upload_inputs(citcom_nn *n, const float *x)
{
	std::vector<__nv_bfloat16> hb((size_t)n->V * NN_CH, __float2bfloat16_rn(0.f));
	for(int v = 0; v < n->V; ++v)
		for(int c = 0; c < NN_IN; ++c)
			hb[(size_t)v * NN_CH + c] = __float2bfloat16_rn(x[(size_t)v * NN_IN + c]);
	if(cudaMemcpyAsync(n->x, hb.data(), hb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, n->h->st) != cudaSuccess ||
	   cudaStreamSynchronize(n->h->st) != cudaSuccess)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "input upload failed");
	return CITCOM_GPU_OK;
}

unsigned long long nn_rand(citcom_nn *n)
{
	n->rng = n->rng * 6364136223846793005ull + 1442695040888963407ull;
	return n->rng >> 17;
}

} // namespace

extern "C" {

int citcom_nn_create(citcom_gpu *h, int level, unsigned seed, int capacity, citcom_nn **out)
{
	TRY(check_handle(h));
	if(!out)
		return fail(h, CITCOM_GPU_ERR_ARG, "null argument");
	*out = nullptr;
	const int lmax = h->L - 1;
	if(level < 0)
		level = lmax - 1;
	if(level < 1 || level >= lmax)
		return fail(h, CITCOM_GPU_ERR_ARG, "warm-start level %d: needs 1 <= level < %d", level, lmax);
	if(capacity < 1)
		return fail(h, CITCOM_GPU_ERR_ARG, "training-set capacity must be positive");
	citcom_nn *n = new citcom_nn();
	n->h = h;
	n->check_every = 1;
	n->lev = level;
	n->r = 1 << (lmax - level);
	n->capacity = capacity;
	n->rng = 0x2545F4914F6CDD1Dull ^ seed;
	const Lvl &Lc = h->lv[level];
	if(nn_create(Lc.nox, Lc.noy, Lc.noz, seed, h->st, &n->net, n->err, sizeof(n->err)) != 0)
	{
		int r = fail(h, CITCOM_GPU_ERR_ARG, "%s", n->err);
		delete n;
		return r;
	}
	n->V = nn_voxels(n->net);
	int r = CITCOM_GPU_OK;
	r = r ? r : nn_alloc(n, &n->xs, (size_t)capacity * n->V * NN_CH);
	r = r ? r : nn_alloc(n, &n->ts, (size_t)capacity * n->V * NN_OUT);
	r = r ? r : nn_alloc(n, &n->x, (size_t)n->V * NN_CH);
	r = r ? r : nn_alloc(n, &n->y, (size_t)n->V * NN_CH);
	for(int l = level; l < lmax && !r; ++l)
		r = nn_alloc(n, &n->Uv[l], (size_t)h->lv[l].neq + 2);
	r = r ? r : nn_alloc(n, &n->Ug, (size_t)h->lv[lmax].neq + 2);
	r = r ? r : nn_alloc(n, &n->Pg, (size_t)h->lv[lmax].nel);
	r = r ? r : nn_alloc(n, &n->work, (size_t)Lc.nno + Lc.noz + 2);
	r = r ? r : nn_alloc(n, &n->Tp, (size_t)h->lv[lmax].nno);
	r = r ? r : nn_alloc(n, &n->dT, (size_t)h->lv[lmax].nno);
	r = r ? r : nn_alloc(n, &n->Up, (size_t)h->lv[lmax].neq + 2);
	r = r ? r : nn_alloc(n, &n->Pp, (size_t)h->lv[lmax].nel);
	if(r != CITCOM_GPU_OK)
	{
		fail(h, r, "%s", n->err);
		citcom_nn_destroy(n);
		return r;
	}
	*out = n;
	return CITCOM_GPU_OK;
}

void citcom_nn_destroy(citcom_nn *n)
{
	if(!n)
		return;
	if(n->h)
	{
		cudaStreamSynchronize(n->h->st);
		if(n->h->warm == n)
			n->h->warm = nullptr;
	}
	nn_destroy(n->net);
	for(void *p : n->allocs)
		cudaFree(p);
	delete n;
}

const char *citcom_nn_error_string(const citcom_nn *n) { return n ? n->err : "null network"; }

int citcom_nn_info(const citcom_nn *n, int info[6])
{
	if(!n || !info)
		return CITCOM_GPU_ERR_ARG;
	const Lvl &Lc = n->h ? n->h->lv[n->lev] : Lvl();
	info[0] = Lc.nox;
	info[1] = Lc.noy;
	info[2] = Lc.noz;
	info[3] = nn_param_count(n->net);
	info[4] = n->count;
	info[5] = n->lev;
	return CITCOM_GPU_OK;
}

int citcom_nn_get_params(citcom_nn *n, float *w)
{
	NTRY(nn_check(n));
	if(!w)
		return nn_fail(n, CITCOM_GPU_ERR_ARG, "null argument");
	return nn_get_params(n->net, w) == 0 ? CITCOM_GPU_OK : nn_fail(n, CITCOM_GPU_ERR_CUDA, "parameter download failed");
}

int citcom_nn_set_params(citcom_nn *n, const float *w)
{
	NTRY(nn_check(n));
	if(!w)
		return nn_fail(n, CITCOM_GPU_ERR_ARG, "null argument");
	return nn_set_params(n->net, w) == 0 ? CITCOM_GPU_OK : nn_fail(n, CITCOM_GPU_ERR_CUDA, "parameter upload failed");
}

int citcom_nn_get_scales(const citcom_nn *n, double s[3])
{
	if(!n || !s)
		return CITCOM_GPU_ERR_ARG;
	s[0] = n->su;
	s[1] = n->sp;
	s[2] = n->mp;
	return n->scaled ? CITCOM_GPU_OK : CITCOM_GPU_ERR_STATE;
}

int citcom_nn_set_scales(citcom_nn *n, const double s[3])
{
	NTRY(nn_check(n));
	if(!s || !(s[0] > 0.0) || !(s[1] > 0.0))
		return nn_fail(n, CITCOM_GPU_ERR_ARG, "scales must be positive");
	n->su = s[0];
	n->sp = s[1];
	n->mp = s[2];
	n->scaled = true;
	return CITCOM_GPU_OK;
}

int citcom_nn_record(citcom_nn *n)
{
	NTRY(nn_check(n));
	citcom_gpu *h = n->h;
	const int lmax = h->L - 1;
	const Lvl &Lf = h->lv[lmax], &Lc = h->lv[n->lev];
	if(!h->visc_ready)
		return nn_fail(n, CITCOM_GPU_ERR_STATE, "no viscosity: record after a Stokes solve");
	__nv_bfloat16 *xs = n->xs + (size_t)n->next * n->V * NN_CH;
	float *ts = n->ts + (size_t)n->next * n->V * NN_OUT;
	const double *Ts = h->T, *Us = h->U, *Ps = h->P;
	if(n->mode == CITCOM_NN_INCREMENT)
	{
		// a sample is the change since the previous record of the same state
		// sequence (no load_state in between); the first record of a sequence
		// only remembers its state
		const bool sample = n->have_prev && n->prev_gen == h->state_gen;
		if(sample)
		{
			launch_lin2(h->st, Lf.nno, n->dT, 1.0, h->T, -1.0, n->Tp);
			launch_lin2(h->st, Lf.neq, n->Ug, 1.0, h->U, -1.0, n->Up);
			launch_lin2(h->st, Lf.nel, n->Pg, 1.0, h->P, -1.0, n->Pp);
			Ts = n->dT;
			Us = n->Ug;
			Ps = n->Pg;
		}
		CK(cudaMemcpyAsync(n->Tp, h->T, sizeof(double) * Lf.nno, cudaMemcpyDeviceToDevice, h->st));
		CK(cudaMemcpyAsync(n->Up, h->U, sizeof(double) * Lf.neq, cudaMemcpyDeviceToDevice, h->st));
		CK(cudaMemcpyAsync(n->Pp, h->P, sizeof(double) * Lf.nel, cudaMemcpyDeviceToDevice, h->st));
		n->have_prev = true;
		n->prev_gen = h->state_gen;
		if(!sample)
			return CITCOM_GPU_OK;
	}
	launch_nn_inputs(h->st, Lf, Lc, n->r, Ts, h->evi[n->lev], xs, n->work);
	if(!n->scaled)
	{
		// output scales from the first recorded sample: RMS velocity dof and
		// RMS pressure deviation, per unit anomaly RMS
		std::vector<double> U(Lf.neq), P(Lf.nel);
		double ss = 0.0;
		if(d2h(h, U.data(), Us, sizeof(double) * Lf.neq) || d2h(h, P.data(), Ps, sizeof(double) * Lf.nel) ||
		   d2h(h, &ss, n->work + Lc.nno + Lc.noz, sizeof(double)) || sync(h))
			return nn_fail(n, CITCOM_GPU_ERR_CUDA, "state download failed");
		const double a = std::sqrt(ss / Lc.nno);
		double uu = 0.0, pm = 0.0, pp = 0.0;
		for(double u : U)
			uu += u * u;
		for(double p : P)
			pm += p;
		pm /= Lf.nel;
		for(double p : P)
			pp += (p - pm) * (p - pm);
		if(!(a > 0.0) || !(uu > 0.0) || !(pp > 0.0))
			return nn_fail(n, CITCOM_GPU_ERR_STATE, "the recorded state has no temperature anomaly or no flow");
		n->su = std::sqrt(uu / Lf.neq) / a;
		n->sp = std::sqrt(pp / Lf.nel) / a;
		n->mp = 0.0;
		n->scaled = true;
	}
	launch_nn_targets(h->st, Lf, Lc, n->r, Us, Ps, n->su, n->sp, n->work, ts);
	n->next = (n->next + 1) % n->capacity;
	if(n->count < n->capacity)
		n->count++;
	if(cudaGetLastError() != cudaSuccess)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "record kernels failed to launch");
	return CITCOM_GPU_OK;
}

int citcom_nn_train(citcom_nn *n, int steps, int batch, double lr, double *loss)
{
	NTRY(nn_check(n));
	if(n->count < 1)
		return nn_fail(n, CITCOM_GPU_ERR_STATE, "the training set is empty");
	if(steps < 1 || batch < 1 || !(lr > 0.0))
		return nn_fail(n, CITCOM_GPU_ERR_ARG, "steps, batch and lr must be positive");
	const float scale = 1.f / ((float)n->V * NN_OUT * batch);
	for(int s = 0; s < steps; ++s)
	{
		nn_zero_grads(n->net);
		for(int b = 0; b < batch; ++b)
		{
			const int i = (int)(nn_rand(n) % (unsigned long long)n->count);
			nn_accumulate(n->net, n->xs + (size_t)i * n->V * NN_CH, n->ts + (size_t)i * n->V * NN_OUT, scale);
		}
		nn_adam(n->net, (float)lr, 0.9f, 0.999f, 1e-8f);
	}
	double l = 0.0;
	if(nn_loss(n->net, &l) != 0)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "training failed: %s", cudaGetErrorString(cudaGetLastError()));
	if(nn_device_error(n->net) != 0)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "training: a tensor-core wait timed out");
	if(loss)
		*loss = l;
	return CITCOM_GPU_OK;
}

int citcom_nn_set_mode(citcom_nn *n, int mode)
{
	NTRY(nn_check(n));
	if(mode != CITCOM_NN_ABSOLUTE && mode != CITCOM_NN_INCREMENT)
		return nn_fail(n, CITCOM_GPU_ERR_ARG, "unknown warm-start mode %d", mode);
	if(n->count > 0 || n->have_prev || n->scaled)
		return nn_fail(n, CITCOM_GPU_ERR_STATE, "the mode must be set before the first record");
	n->mode = mode;
	return CITCOM_GPU_OK;
}

int citcom_nn_set_check_interval(citcom_nn *n, int every)
{
	NTRY(nn_check(n));
	if(every < 1)
		return nn_fail(n, CITCOM_GPU_ERR_ARG, "the check interval must be at least 1");
	n->check_every = every;
	n->guesses = 0;
	n->net_ok = false;
	n->r_ref = 0.0;
	return CITCOM_GPU_OK;
}

int citcom_nn_attach(citcom_nn *n, int on)
{
	NTRY(nn_check(n));
	n->attached = on != 0;
	n->h->warm = n->attached ? n : (n->h->warm == n ? nullptr : n->h->warm);
	return CITCOM_GPU_OK;
}

int citcom_nn_predict(citcom_nn *n, double *U, double *P)
{
	NTRY(nn_check(n));
	citcom_gpu *h = n->h;
	if(!n->scaled)
		return nn_fail(n, CITCOM_GPU_ERR_STATE, "no output scales: record a solution or set the scales first");
	if(!h->visc_ready)
		return nn_fail(n, CITCOM_GPU_ERR_STATE, "no viscosity: call get_system_viscosity or solve first");
	if(n->mode != CITCOM_NN_ABSOLUTE)
		return nn_fail(n, CITCOM_GPU_ERR_STATE, "predict needs the absolute mode (an increment has no state of its own)");
	const Lvl &Lf = h->lv[h->L - 1];
	if(nn_guess(n) != CITCOM_GPU_OK)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "%s", h->err);
	if((U && d2h(h, U, n->Ug, sizeof(double) * Lf.neq)) || (P && d2h(h, P, n->Pg, sizeof(double) * Lf.nel)) || sync(h))
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "guess download failed");
	return nn_device_error(n->net) == 0 ? CITCOM_GPU_OK : nn_fail(n, CITCOM_GPU_ERR_CUDA, "a tensor-core wait timed out");
}

int citcom_nn_forward(citcom_nn *n, const float *x, float *y)
{
	NTRY(nn_check(n));
	if(!x || !y)
		return nn_fail(n, CITCOM_GPU_ERR_ARG, "null argument");
	NTRY(nn_upload_inputs(n, x));
	nn_forward(n->net, n->x, n->y);
	std::vector<float> hy((size_t)n->V * NN_CH);
	if(cudaMemcpyAsync(hy.data(), n->y, hy.size() * sizeof(float), cudaMemcpyDeviceToHost, n->h->st) != cudaSuccess ||
	   cudaStreamSynchronize(n->h->st) != cudaSuccess)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "forward failed: %s", cudaGetErrorString(cudaGetLastError()));
	if(nn_device_error(n->net) != 0)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "forward: a tensor-core wait timed out");
	for(int v = 0; v < n->V; ++v)
		for(int c = 0; c < NN_OUT; ++c)
			y[(size_t)v * NN_OUT + c] = hy[(size_t)v * NN_CH + c];
	return CITCOM_GPU_OK;
}

int citcom_nn_loss_grad(citcom_nn *n, const float *x, const float *t, double *loss, float *grad)
{
	NTRY(nn_check(n));
	if(!x || !t || !loss || !grad)
		return nn_fail(n, CITCOM_GPU_ERR_ARG, "null argument");
	NTRY(nn_upload_inputs(n, x));
	float *dt = n->ts;  // slot 0 of the training set as scratch for the target
	if(cudaMemcpyAsync(dt, t, sizeof(float) * n->V * NN_OUT, cudaMemcpyHostToDevice, n->h->st) != cudaSuccess)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "target upload failed");
	nn_zero_grads(n->net);
	nn_accumulate(n->net, n->x, dt, 1.f / ((float)n->V * NN_OUT));
	if(nn_loss(n->net, loss) != 0 || nn_get_grads(n->net, grad) != 0)
		return nn_fail(n, CITCOM_GPU_ERR_CUDA, "gradient failed: %s", cudaGetErrorString(cudaGetLastError()));
	if(n->count > 0)
		n->count = 0, n->next = 0;  // slot 0 was overwritten
	return nn_device_error(n->net) == 0 ? CITCOM_GPU_OK : nn_fail(n, CITCOM_GPU_ERR_CUDA, "a tensor-core wait timed out");
}

} // extern "C"
