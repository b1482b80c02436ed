// qew_noalloc.cu -- line energy without any device-memory allocation.
//
// qew_objective needs reduction scratch (one partial sum per CTA and a ticket
// counter), which lives in a context created with cudaMalloc. Some callers
// cannot make that call where they need the energy: cudaMalloc and cudaFree
// may synchronise the whole device, which a latency-bound serving loop
// running other streams cannot afford; and a process whose device memory is
// entirely reserved up front (an HBM budget, or another framework's caching
// allocator owning the device) gets out-of-memory from any extra cudaMalloc.
// qew_objective_noalloc serves them: the scratch is a file-scope device array
// that every GPU loading this library holds until the process exits, so the
// entry point itself allocates nothing. The caller passes the inputs and a
// device pointer for the result.
//
// Limits and sharing: one partial per CTA of 256 edges, at most
// QEW_NOALLOC_MAX_N = 4096 * 256 = 2^20 edges; longer lines are rejected with
// QEW_ERR_INVALID. All calls on a device share the one array and it keeps
// the previous call's contents, so the ticket counter is cleared at the start
// of every call (the partials are rewritten before they are read); calls that
// overlap on the GPU (different streams, or host threads) race on the array
// and must be serialised by the caller.
#include <cuda.h>  // driver types only: the two driver calls are resolved at run time

#include <mutex>

#include "qew_internal.cuh"
#include "qew_model_kernels.cuh"

namespace {

constexpr int kNoAllocBS = 256;
constexpr int kNoAllocMaxBlocks = QEW_NOALLOC_MAX_N / kNoAllocBS;  // 4096
constexpr int kMaxDevices = 64;

// [0, 4096): per-CTA partial sums; element 4096 holds the ticket counter.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxBlocks + 32];

std::mutex g_setup_mu;
struct ScratchSlot {
    double *ptr = nullptr;
    unsigned long long ctx_id = 0;  // the context the address belongs to
};
ScratchSlot g_scratch[kMaxDevices];

// Unique id of the calling thread's current CUDA context (cuCtxGetId ids are
// never reused within a process), through driver entry points looked up once.
bool current_context_id(unsigned long long *id) {
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {  // under g_setup_mu
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa{}, qb{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault,
                                             &qa) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) ==
                cudaSuccess &&
            qa == cudaDriverEntryPointSuccess && qb == cudaDriverEntryPointSuccess) {
            get_current = (GetCurrent)a;
            get_id = (GetId)b;
        }
        cudaGetLastError();
        resolved = true;
    }
    CUcontext c = nullptr;
    return get_current && get_id && get_current(&c) == CUDA_SUCCESS && c &&
           get_id(c, id) == CUDA_SUCCESS;
}

// The array's name is only a host-side stand-in: its device address is looked
// up with the device current, once per device and context, and passed to the
// kernel. A device whose context was destroyed and created again (after
// cudaDeviceReset, say) has a new context id, so its address is looked up
// again instead of reusing the old one.
qew_status scratch_address(int device, double **out) {
    if (device < 0 || device >= kMaxDevices) return QEW_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    ScratchSlot &slot = g_scratch[device];
    unsigned long long id = 0;
    bool have_id = current_context_id(&id);
    if (!slot.ptr || !have_id || slot.ctx_id != id) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return QEW_ERR_CUDA;
        }
        if (!have_id) have_id = current_context_id(&id);  // the look-up made the context
        slot.ptr = (double *)p;
        slot.ctx_id = have_id ? id : 0;
    }
    *out = slot.ptr;
    return QEW_OK;
}

}  // namespace

extern "C" qew_status qew_objective_noalloc(const qew_field *field, const double *d_h, int n,
                                            const qew_params *p, double *d_out,
                                            void *cuda_stream) {
    if (!field || !d_h || !p || !d_out || n < 1) return QEW_ERR_INVALID;
    if (n > QEW_NOALLOC_MAX_N) return QEW_ERR_INVALID;  // beyond the static scratch
    int device = -1;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        return QEW_ERR_CUDA;
    }
    if (device != field->device) return QEW_ERR_INVALID;  // make the field's device current
    double *scratch = nullptr;
    QEW_TRY(scratch_address(device, &scratch));
    double *partials = scratch;
    unsigned int *counter = (unsigned int *)(scratch + kNoAllocMaxBlocks);
    cudaStream_t stream = (cudaStream_t)cuda_stream;
    if (cudaMemsetAsync(counter, 0, sizeof(unsigned int), stream) != cudaSuccess) {
        cudaGetLastError();
        return QEW_ERR_CUDA;
    }
    const LineDx dx = make_line_dx(p->physical_size, n);
    const int blocks = (n + kNoAllocBS - 1) / kNoAllocBS;  // <= kNoAllocMaxBlocks
    return qew_dispatch_noise(nullptr, field, [&](auto nz) -> qew_status {
        k_objective<decltype(nz), LineAt, kNoAllocBS><<<blocks, kNoAllocBS, 0, stream>>>(
            n, dx, p->line_tension, p->driving_force, p->model, nz, LineAt{d_h}, partials,
            counter, d_out);
        const cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? QEW_OK : QEW_ERR_CUDA;
    }, n, p->physical_size);
}
