// noalloc.cu -- velocity_at for callers that cannot allocate device memory.
//
// Some host programs own every byte of device memory themselves: a simulation
// framework that reserves one arena up front and forbids allocations inside its
// time-stepping loop, or a process that shares the GPU under a fixed memory
// budget where an allocation failing in mid-run is not acceptable.  Such a
// caller passes its own device buffers for the inputs and the outputs; the
// only other memory this entry point needs -- the per-panel geometry records
// the field kernel reads and its overflow flag -- lives in the file-scope
// device array below, sized for SQBEM_NOALLOC_MAX_PANELS panels (2.3 MB, held
// by every GPU that loads the library until the process exits).
//
// The array is shared by every call: each call overwrites the records and
// clears the flag before its kernels run, so calls that overlap on the GPU
// (issued on different streams without ordering) race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "assemble.cuh"
#include "common.cuh"
#include "sqbem.h"

namespace sqbem {
namespace {

constexpr int NA_MAXP = SQBEM_NOALLOC_MAX_PANELS;
constexpr size_t NA_FLAG_OFFSET = (size_t)NA_MAXP * sizeof(PanelRec);
constexpr size_t NA_BYTES = NA_FLAG_OFFSET + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

std::mutex g_na_mu;
void* g_na_addr[64] = {};

// Device address of the scratch array on the current device.  The name of the
// array is only a host-side stand-in; the address is looked up once per device
// (on that device's first call) and cached.
unsigned char* scratch_address() {
    int dev = 0;
    CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) fail(SQBEM_ERR_ARG, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            fail(SQBEM_ERR_CUDA, "cudaGetSymbolAddress of the no-allocation scratch failed: %s", cudaGetErrorString(e));
        g_na_addr[dev] = p;
    }
    return static_cast<unsigned char*>(g_na_addr[dev]);
}

// Panel records from vertices with the operation order and rounding of the host
// geometry (Mesh::geometry, mesh.hpp:61-72): round-to-nearest products and sums
// without contraction, IEEE sqrt and division, so the records equal the ones the
// allocating entry point builds on the host.
__global__ void geometry_kernel(int P, const double* __restrict__ V, PanelRec* __restrict__ out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const double* v = V + 9 * (long long)p;
    const double ax = v[0], ay = v[1], az = v[2];
    const double e1x = __dsub_rn(v[3], ax), e1y = __dsub_rn(v[4], ay), e1z = __dsub_rn(v[5], az);
    const double e2x = __dsub_rn(v[6], ax), e2y = __dsub_rn(v[7], ay), e2z = __dsub_rn(v[8], az);
    const double cx = __dsub_rn(__dmul_rn(e1y, e2z), __dmul_rn(e1z, e2y));
    const double cy = __dsub_rn(__dmul_rn(e1z, e2x), __dmul_rn(e1x, e2z));
    const double cz = __dsub_rn(__dmul_rn(e1x, e2y), __dmul_rn(e1y, e2x));
    const double nn = __dadd_rn(__dadd_rn(__dmul_rn(cx, cx), __dmul_rn(cy, cy)), __dmul_rn(cz, cz));
    const double area = __dmul_rn(0.5, __dsqrt_rn(nn));
    const double inv = __ddiv_rn(1.0, __dmul_rn(2.0, area));
    PanelRec& r = out[p];
    for (int k = 0; k < 9; ++k) r.v[k] = v[k];
    r.n[0] = __dmul_rn(inv, cx);
    r.n[1] = __dmul_rn(inv, cy);
    r.n[2] = __dmul_rn(inv, cz);
    const double third = 1.0 / 3;
    r.c[0] = __dmul_rn(third, __dadd_rn(__dadd_rn(v[0], v[3]), v[6]));
    r.c[1] = __dmul_rn(third, __dadd_rn(__dadd_rn(v[1], v[4]), v[7]));
    r.c[2] = __dmul_rn(third, __dadd_rn(__dadd_rn(v[2], v[5]), v[8]));
    r.area = area;
    r.h = __dsqrt_rn(__dmul_rn(2.0, area));
    r.pad = 0.0;
}

}  // namespace
}  // namespace sqbem

using namespace sqbem;

extern "C" int sqbem_velocity_at_noalloc(int P, const double* V, const double* u, const double* f, double mu,
                                         int npts, const double* pts, double* out, int precision, void* stream) {
    return guarded([&] {
        if (P < 0 || npts < 0 || !(mu > 0) || (P > 0 && (!V || !u || !f)) || (npts > 0 && (!pts || !out)) ||
            (precision != SQBEM_FP64 && precision != SQBEM_MIXED))
            fail(SQBEM_ERR_ARG, "velocity_at_noalloc: bad arguments");
        if (P > NA_MAXP)
            fail(SQBEM_ERR_ARG, "velocity_at_noalloc: %d panels exceed the no-allocation limit of %d panels", P,
                 NA_MAXP);
        if (npts == 0) return;
        require_device();
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        unsigned char* scratch = scratch_address();
        PanelRec* recs = reinterpret_cast<PanelRec*>(scratch);
        int* overflow = reinterpret_cast<int*>(scratch + NA_FLAG_OFFSET);
        CUDA_CHECK(cudaMemsetAsync(overflow, 0, sizeof(int), st));
        if (P > 0) LAUNCH(geometry_kernel, ceil_div(P, 128), 128, 0, st, P, V, recs);
        FieldJob job;
        job.pts = pts;
        job.npts = npts;
        job.panels = recs;
        job.P = P;
        job.u = u;
        job.f = f;
        job.sscale = 1.0 / (EIGHT_PI * mu);
        job.dscale = -1.0 / EIGHT_PI;
        job.out = out;
        job.overflow = overflow;
        job.mixed = precision == SQBEM_MIXED;
        field_eval(job, st);
        int h_ovf = 0;
        CUDA_CHECK(cudaMemcpyAsync(&h_ovf, overflow, sizeof(int), cudaMemcpyDeviceToHost, st));
        count_d2h(sizeof(int));
        CUDA_CHECK(cudaStreamSynchronize(st));
        if (h_ovf) fail(SQBEM_ERR_ARG, "velocity_at_noalloc: a point has more than 256 near panels");
    });
}
