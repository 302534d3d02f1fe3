// fvm_rhs_noalloc: fvm_eqs! for callers that must not allocate device memory.
//
// fvm_rhs with device arrays in the caller's numbering stages u and du through two work
// vectors in the library's internal numbering, and allocates them with cudaMalloc the first
// time.  Some callers cannot let that happen: real-time loops whose allocator is frozen after
// start-up, and hosts that hand all device memory to their own pool, where a cudaMalloc
// behind the pool's back fails or fragments it.  This entry point uses a fixed scratch area
// compiled into the library instead, so a call makes no cudaMalloc, cudaFree or other
// allocating call.
//
// The scratch lives in a file-scope __device__ array sized for FVM_NOALLOC_MAX_POINTS points
// (2 x 262,144 doubles = 4 MiB).  Every GPU that loads the library holds it until the
// process exits.  Host code cannot use the array's name as a device address, so the device
// address is looked up once per device with cudaGetSymbolAddress, with that device current,
// on the first call made on that device.
#include "fvm_internal.h"

#include <mutex>

namespace {

__device__ __align__(256) double g_rhs_scratch[2 * FVM_NOALLOC_MAX_POINTS];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of g_rhs_scratch on the current device (looked up once per device).
double* scratch_for_current_device() {
    int dev = -1;
    FVM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) fvm::fail(FVM_ERR_INVALID_ARGUMENT, "device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_rhs_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            fvm::fail(FVM_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        }
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    return g_scratch_addr[dev];
}

}  // namespace

extern "C" int fvm_rhs_noalloc(fvm_problem* p, const double* u, double* du, double t, void* stream) {
    return fvm::guard_call([&] {
        if (!p || !u || !du) fvm::fail(FVM_ERR_INVALID_ARGUMENT, "NULL argument");
        const fvm_mesh* m = p->mesh;
        int dev = -1;
        FVM_CUDA(cudaGetDevice(&dev));
        if (dev != m->device)
            fvm::fail(FVM_ERR_INVALID_ARGUMENT, "fvm_rhs_noalloc: the mesh was created on device " +
                                               std::to_string(m->device) + ", the current device is " +
                                               std::to_string(dev));
        if (m->np > FVM_NOALLOC_MAX_POINTS)
            fvm::fail(FVM_ERR_INVALID_ARGUMENT, "fvm_rhs_noalloc handles at most " +
                                                    std::to_string(FVM_NOALLOC_MAX_POINTS) + " points; this mesh has " +
                                                    std::to_string(m->np) + " (use fvm_rhs)");
        if (p->conditions_only)
            fvm::fail(FVM_ERR_INVALID_ARGUMENT, "this problem carries a template's conditions only");
        if (!p->linear && !p->tri_ready)
            fvm::fail(FVM_ERR_INVALID_ARGUMENT,
                      "fvm_rhs_noalloc: this problem's per-triangle data is prepared by its first fvm_rhs call; "
                      "make one fvm_rhs call before using the no-allocation entry point");
        cudaStream_t s = (cudaStream_t)stream;
        double* scratch = scratch_for_current_device();
        double* u_int = scratch;                           // u in the internal numbering
        double* du_int = scratch + FVM_NOALLOC_MAX_POINTS;  // du in the internal numbering
        // every entry of both halves is written before it is read, so stale contents from an
        // earlier call never leak into this one
        fvm::launch_permute_in(m->d_perm.as<int32_t>(), u, u_int, m->np, s);
        fvm::problem_rhs_internal(p, u_int, du_int, false, s, false, t);
        fvm::launch_permute_out(m->d_perm.as<int32_t>(), du_int, du, m->np, s);
        FVM_CUDA(cudaGetLastError());
        return FVM_OK;
    });
}
