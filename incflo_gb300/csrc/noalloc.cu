// gbp_nodal_divergence_noalloc: the nodal divergence of gbp_nodal_divergence for callers that cannot
// allocate device memory: a host application whose device memory belongs to another framework's
// allocator (which may own the whole memory pool, or forbid cudaMalloc / cudaFree while it runs), or an
// embedding such as a solver plugin that may not create a plan. It needs no plan: it reads the
// caller's velocity, writes the caller's output, and keeps its only scratch (per-block partial sums
// and two scalars) in the file-scope device array below, which every GPU that loads this library
// holds until the process exits.
//
// Limits and rules:
//  - scratch holds kMaxBlocks per-block partial sums: at most 65536 blocks of 32 x 4 x 4 nodes, i.e.
//    about 33.5 million nodes (256^3 fits; larger grids are rejected with GBP_BAD_ARG);
//  - the first call on a device (and the first call after that device's context was reset) looks up
//    the array's device address (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture;
//  - every call shares the one array: calls that overlap on the GPU (different streams, or another
//    host thread) race on it; serialise them;
//  - each call ends by reading the max norm back to the host, so it synchronises the stream it is
//    given.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "gbp_internal.cuh"

namespace gbp {

namespace {

constexpr int kMaxBlocks = 65536;
constexpr int kMaxDevices = 64;
constexpr int BX = 32, BY = 4, BZ = 4;

// [0, kMaxBlocks): per-block sums of the weak right-hand side; [kMaxBlocks]: the consistency
// shift; [kMaxBlocks + 1]: the max norm (as ordered bits)
static __device__ __align__(256) double g_noalloc_scratch[kMaxBlocks + 8];

// the scratch address per device, with the context it was looked up in: a device reset creates a new
// context (and reloads this module), after which the address is looked up again
std::mutex g_mu;
double* g_dev_scratch[kMaxDevices] = {};
CUcontext g_dev_ctx[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
CtxGetCurrentFn ctx_get_current()
{
    static CtxGetCurrentFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrentFn>(p);
    });
    return fn;
}

__device__ __forceinline__ double a4v(const gbp_array4& a, int i, int j, int k, int n)
{
    return a.data[(long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride + (long long)(k - a.lo[2]) * a.kstride +
                  (long long)n * a.nstride];
}
__device__ __forceinline__ double* a4q(const gbp_array4& a, int i, int j, int k)
{
    return a.data + (long long)(i - a.lo[0]) + (long long)(j - a.lo[1]) * a.jstride + (long long)(k - a.lo[2]) * a.kstride;
}

struct DivArgs {
    gbp_array4 vel, out;
    int inflow_lo[3], inflow_hi[3];
    double cf[3];
};

// Weak divergence per node from per-cell fluxes staged in shared memory (the construction of the
// plan-based right-hand-side kernel), written as -g/V to every node 0..n of the caller's array;
// per-block sums of g over the unique nodes go to the scratch.
__global__ void __launch_bounds__(BX* BY* BZ) k_div_noalloc(NodalGeom g, DivArgs a, double* __restrict__ part)
{
    __shared__ double F[3][BZ + 1][BY + 1][BX + 1];
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY, z0 = blockIdx.z * BZ;
    const int tid = threadIdx.x + BX * (threadIdx.y + BY * threadIdx.z);
    constexpr int NC = (BX + 1) * (BY + 1) * (BZ + 1);
    for (int q = tid; q < NC; q += BX * BY * BZ) {
        const int cx = q % (BX + 1), cy = (q / (BX + 1)) % (BY + 1), cz = q / ((BX + 1) * (BY + 1));
        int cell[3] = {x0 - 1 + cx, y0 - 1 + cy, z0 - 1 + cz};
        int nout = 0, dout = -1;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int ci = cell[d];
            if (g.per[d]) {
                ci = ((ci % g.n[d]) + g.n[d]) % g.n[d];
            } else if (ci < -1 || ci > g.n[d]) {
                nout += 2;  // beyond the one ghost layer: no flux, and never read
            } else if (ci == -1 || ci == g.n[d]) {
                ++nout;
                dout = d;
            }
            cell[d] = ci;
        }
        double f[3] = {0.0, 0.0, 0.0};
        if (nout == 0) {
#pragma unroll
            for (int d = 0; d < 3; ++d) f[d] = a.cf[d] * a4v(a.vel, cell[0], cell[1], cell[2], d);
        } else if (nout == 1) {
            const int inflow = cell[dout] < 0 ? a.inflow_lo[dout] : a.inflow_hi[dout];
            if (inflow) f[dout] = a.cf[dout] * a4v(a.vel, cell[0], cell[1], cell[2], dout);
        }
        F[0][cz][cy][cx] = f[0];
        F[1][cz][cy][cx] = f[1];
        F[2][cz][cy][cx] = f[2];
    }
    __syncthreads();
    const int tx = threadIdx.x, ty = threadIdx.y, tz = threadIdx.z;
    const int i = x0 + tx, j = y0 + ty, k = z0 + tz;
    double gv = 0.0;
    // all nodes 0..n: the periodic duplicate node n carries the value of node 0 and is left out of the sums
    if (i <= g.n[0] && j <= g.n[1] && k <= g.n[2]) {
        if (!node_is_dirichlet(g, i, j, k)) {
            double dx = 0.0, dy = 0.0, dz = 0.0;
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
                for (int bq = 0; bq < 2; ++bq) {
                    dx += F[0][tz + c][ty + bq][tx + 1] - F[0][tz + c][ty + bq][tx];
                    dy += F[1][tz + c][ty + 1][tx + bq] - F[1][tz + c][ty][tx + bq];
                    dz += F[2][tz + 1][ty + c][tx + bq] - F[2][tz][ty + c][tx + bq];
                }
            gv = -((dx + dy) + dz);
        }
        const int iu = (g.per[0] && i == g.n[0]) ? 0 : i;
        const int ju = (g.per[1] && j == g.n[1]) ? 0 : j;
        const int ku = (g.per[2] && k == g.n[2]) ? 0 : k;
        *a4q(a.out, i, j, k) = -gv * node_inv_volume(g, iu, ju, ku);
        if (iu != i || ju != j || ku != k) gv = 0.0;
    } else {
        gv = 0.0;
    }
    const double t = block_sum_all(gv);
    if (tid == 0) part[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = t;
}

// shift = sum(g) / sum(V) in a fixed order (singular boundary sets only)
__global__ void __launch_bounds__(1024) k_fold_noalloc(const double* __restrict__ part, int nparts, double vtot,
                                                       double* __restrict__ shift)
{
    double acc = 0.0;
    for (int t = threadIdx.x; t < nparts; t += blockDim.x) acc += part[t];
    acc = block_sum_all(acc);
    if (threadIdx.x == 0) *shift = acc / vtot;
}

// out += shift (strong form of g -= V shift) on every node; max |out| over the unique nodes
__global__ void __launch_bounds__(256) k_shift_norm_noalloc(NodalGeom g, gbp_array4 out, const double* __restrict__ shift,
                                                            int apply_shift, unsigned long long* norm)
{
    const double c = apply_shift ? *shift : 0.0;
    const int n0 = g.n[0] + 1, n1 = g.n[1] + 1, n2 = g.n[2] + 1;
    const long long nxy = (long long)n0 * n1, total = nxy * n2;
    double nv = 0.0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t / nxy);
        const long long rem = t - (long long)k * nxy;
        const int j = (int)(rem / n0);
        const int i = (int)(rem - (long long)j * n0);
        double* p = a4q(out, i, j, k);
        const double v = *p + c;
        *p = v;
        const bool dup = (g.per[0] && i == g.n[0]) || (g.per[1] && j == g.n[1]) || (g.per[2] && k == g.n[2]);
        if (!dup && !node_is_dirichlet(g, i, j, k)) nv = nanmax(nv, fabs(v));
    }
    nv = block_max(nv);
    if (threadIdx.x == 0) atomic_max_nonneg(norm, nv);
}

}  // namespace

}  // namespace gbp

using namespace gbp;

extern "C" int gbp_nodal_divergence_noalloc(const gbp_geometry* geom, const int bc_lo[3], const int bc_hi[3],
                                            const gbp_array4* vel, int use_inflow, gbp_array4* div_out,
                                            double* max_norm, void* stream)
{
    if (!geom || !bc_lo || !bc_hi || !vel || !vel->data || !div_out || !div_out->data || !max_norm) {
        set_error("gbp_nodal_divergence_noalloc: null argument");
        return GBP_BAD_ARG;
    }
    NodalGeom g;
    memset(&g, 0, sizeof(g));
    bool singular = true;
    for (int d = 0; d < 3; ++d) {
        const int n = geom->n_cell[d];
        const double h = n > 0 ? (geom->prob_hi[d] - geom->prob_lo[d]) / n : 0.0;
        if (n < 2 || !(h > 0.0) || (bc_lo[d] == GBP_BC_PERIODIC) != (bc_hi[d] == GBP_BC_PERIODIC) ||
            bc_lo[d] < GBP_BC_PERIODIC || bc_lo[d] > GBP_BC_INFLOW || bc_hi[d] < GBP_BC_PERIODIC ||
            bc_hi[d] > GBP_BC_INFLOW) {
            set_error("gbp_nodal_divergence_noalloc: bad geometry or boundary types");
            return GBP_BAD_ARG;
        }
        g.n[d] = n;
        g.h[d] = h;
        g.per[d] = bc_lo[d] == GBP_BC_PERIODIC;
        g.nu[d] = g.per[d] ? n : n + 1;
        g.dlo[d] = !g.per[d] && bc_lo[d] == GBP_BC_DIRICHLET;
        g.dhi[d] = !g.per[d] && bc_hi[d] == GBP_BC_DIRICHLET;
        if (g.dlo[d] || g.dhi[d]) singular = false;
    }
    g.vol = g.h[0] * g.h[1] * g.h[2];
    g.ivol = 1.0 / g.vol;
    // argument layout: velocity over the valid cells (+1 ghost across inflow faces), output nodes 0..n
    for (int d = 0; d < 3; ++d) {
        // one ghost cell on each side that is an inflow face (read only when use_inflow is set)
        const int glo = (use_inflow && bc_lo[d] == GBP_BC_INFLOW) ? 1 : 0;
        const int ghi = (use_inflow && bc_hi[d] == GBP_BC_INFLOW) ? 1 : 0;
        if (vel->ncomp < 3 || vel->lo[d] > -glo || vel->hi[d] < g.n[d] - 1 + ghi || div_out->lo[d] > 0 ||
            div_out->hi[d] < g.n[d]) {
            set_error("gbp_nodal_divergence_noalloc: vel must cover the valid cells (3 components, one ghost cell "
                      "across each inflow face) and div_out nodes 0..n");
            return GBP_BAD_ARG;
        }
    }
    const dim3 grid((g.n[0] + 1 + BX - 1) / BX, (g.n[1] + 1 + BY - 1) / BY, (g.n[2] + 1 + BZ - 1) / BZ);
    const long long nblocks = (long long)grid.x * grid.y * grid.z;
    if (nblocks > kMaxBlocks) {
        set_error("gbp_nodal_divergence_noalloc: grid exceeds the static scratch (at most 65536 blocks of 32x4x4 "
                  "nodes, about 33.5 million nodes)");
        return GBP_BAD_ARG;
    }
    // once per device, with that device current: the device address of the scratch array
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("gbp_nodal_divergence_noalloc: device ordinal out of range");
        return GBP_BAD_ARG;
    }
    // cudaFree(0) makes the device's primary context current without allocating, so that the context
    // key below is the one the launches use
    e = cudaFree(nullptr);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFree(nullptr) (context initialisation)");
    CUcontext ctx = nullptr;
    if (auto fn = ctx_get_current()) {
        if (fn(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    }
    double* scr = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_dev_scratch[dev] || g_dev_ctx[dev] != ctx) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
            g_dev_scratch[dev] = static_cast<double*>(p);
            g_dev_ctx[dev] = ctx;
        }
        scr = g_dev_scratch[dev];
    }
    const cudaStream_t st = (cudaStream_t)stream;
    DivArgs a{};
    a.vel = *vel;
    a.out = *div_out;
    for (int d = 0; d < 3; ++d) {
        a.inflow_lo[d] = use_inflow && bc_lo[d] == GBP_BC_INFLOW;
        a.inflow_hi[d] = use_inflow && bc_hi[d] == GBP_BC_INFLOW;
    }
    a.cf[0] = 0.25 * g.h[1] * g.h[2];
    a.cf[1] = 0.25 * g.h[0] * g.h[2];
    a.cf[2] = 0.25 * g.h[0] * g.h[1];
    unsigned long long* dnorm = reinterpret_cast<unsigned long long*>(scr + kMaxBlocks + 1);
    // the norm word accumulates with atomicMax: it must start at zero on every call
    e = cudaMemsetAsync(dnorm, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(noalloc norm)");
    k_div_noalloc<<<grid, dim3(BX, BY, BZ), 0, st>>>(g, a, scr);
    const double vtot = (double)g.n[0] * g.h[0] * (double)g.n[1] * g.h[1] * (double)g.n[2] * g.h[2];
    if (singular) k_fold_noalloc<<<1, 1024, 0, st>>>(scr, (int)nblocks, vtot, scr + kMaxBlocks);
    const long long nodes = (long long)(g.n[0] + 1) * (g.n[1] + 1) * (g.n[2] + 1);
    const unsigned nb = (unsigned)((nodes + 255) / 256 < 1184 ? (nodes + 255) / 256 : 1184);
    k_shift_norm_noalloc<<<nb, 256, 0, st>>>(g, *div_out, scr + kMaxBlocks, singular ? 1 : 0, dnorm);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "noalloc divergence launch");
    unsigned long long bits = 0;
    e = cudaMemcpyAsync(&bits, dnorm, sizeof(bits), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(noalloc norm)");
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize(noalloc)");
    memcpy(max_norm, &bits, sizeof(double));
    return GBP_OK;
}
