// cg_common.cuh — shared pieces of libchmy_gb300: context, error plumbing, device field views.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>

#include "../../include/chmy_gb300.h"

struct cg_graph_entry {
    std::string key;            // bytes of the launch arguments the graph was captured with
    cudaGraphExec_t exec = nullptr;
};

struct cg_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    // reduction scratch: per-field 64-bit max slots (device) and their host mirror (pinned)
    unsigned long long* d_red = nullptr;
    unsigned long long* h_red = nullptr;
    static constexpr int kRedSlots = 64;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    char err[512] = {0};
    cg_graph_entry graphs[8];
    int graph_next = 0;
    // FP32 work arrays of the defect-correction solver (allocated on first use)
    void* dc_pool = nullptr;
    size_t dc_pool_bytes = 0;
    // numbered scratch buffers of the time-stepping loops (grown on demand, freed by cg_destroy)
    // slots: 0 thermal partner, 1 SIA D, 2 PT-diffusion partners, 3 SIA ensemble,
    // 4 PT-diffusion defect-correction pool, 5 SIA reverse step, 6 SIA reverse sweep over a tape,
    // 7 SIA ensemble reverse sweep, 8 explicit-diffusion reverse sweep, 9 thermal-step adjoint,
    // 10 the wait flag of the TMA-fed PT-diffusion iteration
    static constexpr int kScratchSlots = 11;
    void* scratch[kScratchSlots] = {};
    size_t scratch_bytes[kScratchSlots] = {};
};

// Device scratch buffer `slot` of at least `bytes` (reallocated when too small; contents are
// not preserved across growth). Sets *rc on failure and returns NULL.
void* cg_scratch(cg_ctx* ctx, int slot, size_t bytes, int* rc);
// The wait flag of the TMA-fed kernels (scratch slot 10), cleared on the context's stream: a
// kernel whose bounded wait for staged data ran out sets it. cg_tma_check reads it after a run
// (synchronising the stream) and reports CG_ERR_TIMEOUT for `what` when it is set.
int* cg_tma_flag(cg_ctx* ctx, int* rc);
int cg_tma_check(cg_ctx* ctx, int* flag, const char* what);

// Launch layouts chosen by timing (autotuner): a process-wide cache keyed by problem shape.
// CG_AUTOTUNE=0 in the environment turns the timing off (the launchers' fixed rules apply).
struct cg_tune_cfg {
    int seg;      // rows (2D) or planes (3D) per segment; 0 = the launcher's rule
    int variant;  // kernel variant (3D: block shape)
};
bool cg_autotune_enabled();
// CG_TUNE_VERBOSE=1: the autotuners print every candidate's time to stderr
bool cg_tune_verbose();
bool cg_tune_lookup(const std::string& key, cg_tune_cfg* out);
// CG_MARCH_LAYOUT=<segment length>:<variant> in the environment: the layout to use instead of
// the autotuner's (profiling of one layout); false when unset or malformed.
bool cg_tune_forced(cg_tune_cfg* out);
void cg_tune_store(const std::string& key, const cg_tune_cfg& cfg);
// CG_BLOCK=<threads along x>x<threads along y> in the environment (read on every call): the
// block shape of the per-point kernels instead of the autotuner's; false when unset or not a
// valid shape (x a multiple of 32, x * y from 64 to 1024).
bool cg_block_forced(dim3* out);

// Programmatic dependent launch. A kernel launched by cg_launch(..., dep = true) may be
// scheduled while the kernel before it on the stream is still running; it calls cg_dep_wait()
// before its first global-memory access, which returns once that kernel has completed and its
// writes are visible. A kernel that calls cg_dep_wait() runs unchanged when launched the
// ordinary way (the wait returns at once). cg_dep_release() lets the next dependent launch be
// scheduled before this grid ends. CG_PDL=0 in the environment turns the overlap off.
__device__ __forceinline__ void cg_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void cg_dep_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
bool cg_pdl_enabled();
// bc!(V) folded into the velocity reads of the 2D marching kernel (one boundary-condition
// launch per run of PT iterations); CG_BC_FOLD=0 in the environment launches it every iteration.
bool cg_bc_fold_enabled();
// The fused single-pass PT-diffusion iteration (3D FP32); CG_PTDIFF_FUSED=0 keeps the
// two-kernel form.
bool cg_ptdiff_fused_enabled();
// The SIA ensemble as one persistent cooperative launch (CG_SIA_PERSISTENT=1) instead of one
// launch per phase replayed from a CUDA graph (the default, measured faster).
bool cg_sia_persistent_enabled();
// CG_SIA_TILE_ROWS=4|8|16: the SIA ensemble's tile height (rows of 32-point tiles) instead of the
// autotuned one (0 when unset); the results do not depend on it.
int cg_sia_tile_rows_forced();
// Grid barriers of the persistent SIA ensemble kernel: the time limit of every wait
// (CG_SIA_BARRIER_LIMIT_MS, default 2000 ms) and a number of arrivals that the barrier expects
// beyond the grid's blocks (CG_SIA_BARRIER_WITHHELD, default 0). A withheld arrival never
// comes, so every wait runs out: the failure-detection test uses this to check that the kernel
// returns on its limit and the call reports CG_ERR_TIMEOUT.
struct cg_barrier_cfg {
    unsigned long long limit_ns = 2000000000ull;
    int withheld = 0;
};
cg_barrier_cfg cg_sia_barrier_cfg();
// Waits of the TMA-fed kernels: the time limit of every wait (CG_TMA_WAIT_LIMIT_MS, default
// 2000 ms) and a ring plane whose copies the producer does not issue (CG_TMA_WITHHOLD_PLANE,
// default none), so that a test can make the consumers' waits run out without a fault: the
// kernel returns and the call reports CG_ERR_TIMEOUT. Read on every call.
struct cg_tma_cfg {
    unsigned long long limit_ns = 2000000000ull;
    int withhold = -1;
};
cg_tma_cfg cg_tma_wait_cfg();

template <class... P, class... A>
inline cudaError_t cg_launch(void (*kern)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool dep,
                             A&&... args) {
    if (!dep || !cg_pdl_enabled()) {
        kern<<<grid, block, smem, st>>>(std::forward<A>(args)...);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

// bc! over a batch of fields (one launch); dep = true launches it as a dependent launch.
int cg_bc_apply_impl(cg_ctx* ctx, const cg_grid* grid, int nfields, const cg_field* fields, const cg_bc* bcs,
                     bool dep = false);

namespace cgk {

// Arithmetic with explicit round-to-nearest and no contraction into FMA: every operation
// rounds once, in the order the CPU oracle (built with -ffp-contract=off) evaluates it, so the
// marching kernel matches it bitwise and a value recomputed at a segment edge rounds exactly
// like the owner's copy.
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return __fma_rn(a, b, c); }
// 1/x correctly rounded: the same value as the IEEE division 1/x, with fewer instructions
__device__ __forceinline__ float rrcp(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rrcp(double x) { return __drcp_rn(x); }

__device__ __forceinline__ unsigned long long bits_of(double d) { return (unsigned long long)__double_as_longlong(d); }
__device__ __forceinline__ unsigned long long bits_of(float f) { return (unsigned long long)(unsigned)__float_as_int(f); }

// Largest of the block's `bits` into *slot with one atomicMax. Every thread of the block
// calls it. Values are >= 0 (D, or |x|), so the bit patterns order like the values; a NaN orders above every
// number, as it does in an atomicMax per cell.
__device__ __forceinline__ void block_max_bits(unsigned long long bits, unsigned long long* slot) {
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ unsigned long long part[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(FULL, bits, o);
        bits = other > bits ? other : bits;
    }
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthreads = blockDim.x * blockDim.y * blockDim.z;
    const int lane = tid & 31, warp = tid >> 5, nwarps = (nthreads + 31) >> 5;
    if (lane == 0) part[warp] = bits;
    __syncthreads();
    if (warp == 0) {
        bits = lane < nwarps ? part[lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(FULL, bits, o);
            bits = other > bits ? other : bits;
        }
        if (lane == 0 && bits) atomicMax(slot, bits);
    }
}

// Mean time (ms) of three launches after one untimed launch, with CUDA events on `st`;
// -1 if a launch fails (the autotuners' measurement).
template <class F>
inline float time_launches(F&& launch, cudaStream_t st) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return -1.f;
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return -1.f;
    }
    float ms = -1.f;
    if (launch() == cudaSuccess && cudaEventRecord(a, st) == cudaSuccess) {
        bool ok = true;
        for (int r = 0; r < 3 && ok; ++r) ok = launch() == cudaSuccess;
        if (ok && cudaEventRecord(b, st) == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess)
            cudaEventElapsedTime(&ms, a, b);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms;
}

// A device FunctionField (cg_function) in the field precision.
template <class T>
struct FnDev {
    int kind;
    T p[8];
};

// coord(grid, loc, I) (src/Grids/uniform_axis.jl): Vertex muladd(I-1, Δ, o), Center
// muladd(I-1, Δ, muladd(0.5, Δ, o)); muladd is a fused multiply-add, as on the CPU.
template <class T>
__device__ __forceinline__ T grid_coord(T org, T dx, int I, bool vertex) {
    const T o = vertex ? org : rfma(T(0.5), dx, org);
    return rfma(T(I - 1), dx, o);
}

// func(x...) of a device FunctionField at the point x (cg_function's forms; every operation
// rounded once, left to right, as the CPU evaluates the Julia expression).
template <class T>
__device__ __forceinline__ T fn_eval(const FnDev<T>& f, int nd, const T* x) {
    if (f.kind == CG_FN_CONST) return f.p[0];
    if (f.kind == CG_FN_BALL) {
        T r2 = rmul(rsub(x[0], f.p[0]), rsub(x[0], f.p[0]));
        for (int d = 1; d < nd; ++d) r2 = radd(r2, rmul(rsub(x[d], f.p[d]), rsub(x[d], f.p[d])));
        return r2 < rmul(f.p[3], f.p[3]) ? f.p[4] : f.p[5];
    }
    if (f.kind == CG_FN_AFFINE) {
        T v = f.p[0];
        for (int d = 0; d < nd; ++d) v = radd(v, rmul(f.p[1 + d], x[d]));
        return v;
    }
    return T(0);
}

// Block shapes (threads along x, along y) the per-point kernels are timed over. Each thread
// computes one point whatever the shape, so every shape gives the same bits.
constexpr int kBlockShapes[7][2] = {{32, 8}, {32, 4}, {64, 4}, {128, 2}, {32, 16}, {64, 8}, {128, 4}};

// The block shape of a per-point kernel: CG_BLOCK when set, else the fastest of kBlockShapes for
// `key` (timed once per process with `launch(block)`, which must leave no state the caller
// relies on changed), else 32 x 8 when the autotuner is off. `name` labels the verbose output.
template <class F>
inline dim3 tune_block(const char* name, const std::string& key, F&& launch, cudaStream_t st) {
    dim3 b(32, 8);
    if (cg_block_forced(&b)) return b;
    if (!cg_autotune_enabled()) return b;
    cg_tune_cfg c{0, 0};
    if (cg_tune_lookup(key, &c)) return dim3((unsigned)c.seg, (unsigned)c.variant);
    float best = 1e30f;
    for (const auto& sh : kBlockShapes) {
        const dim3 cand((unsigned)sh[0], (unsigned)sh[1]);
        const float t = time_launches([&] { return launch(cand); }, st);
        if (cg_tune_verbose())
            std::fprintf(stderr, "%s tune: block %dx%d: %.1f us\n", name, sh[0], sh[1], t >= 0.f ? 1e3f * t / 3 : -1.f);
        if (t >= 0.f && t < best) {
            best = t;
            b = cand;
        }
    }
    cudaGetLastError();
    cg_tune_store(key, cg_tune_cfg{(int)b.x, (int)b.y});
    return b;
}

}  // namespace cgk

// Record an error message on ctx and return `code`.
int cg_fail(cg_ctx* ctx, int code, const char* fmt, ...);

#define CG_CUDA(ctx, call)                                                                       \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) return cg_fail((ctx), CG_ERR_CUDA, "%s: %s (%s:%d)", #call,      \
                                              cudaGetErrorString(e_), __FILE__, __LINE__);       \
    } while (0)

#define CG_CHECK_LAUNCH(ctx) CG_CUDA(ctx, cudaGetLastError())

// Device view of a field: `p` points at logical index (0,0,0); element (i,j,k) is
// p[i + j*s1 + k*s2]. Logical indices -1 .. n+2 are inside the padded allocation (H >= 1).
template <class T>
struct DF {
    T* __restrict__ p;
    long s1, s2;
    __host__ __device__ __forceinline__ T& operator()(int i, int j, int k) const {
        return p[i + (long)j * s1 + (long)k * s2];
    }
    __host__ __device__ __forceinline__ T* ptr(int i, int j, int k) const {
        return p + i + (long)j * s1 + (long)k * s2;
    }
};

// Offset (elements) of logical index 0 from the allocation start.
inline long cg_origin_offset(const cg_field& f) {
    long off = 0;
    for (int d = 0; d < f.ndim; ++d) off += (long)(2 * f.halo[d] - 1) * f.stride[d];
    return off;
}

template <class T>
inline DF<T> cg_view(const cg_field& f) {
    DF<T> v;
    v.p = static_cast<T*>(f.data) + cg_origin_offset(f);
    v.s1 = f.ndim > 1 ? (long)f.stride[1] : 0;
    v.s2 = f.ndim > 2 ? (long)f.stride[2] : 0;
    return v;
}

// Validate a field against the expected dtype, ndim and per-dim location on `grid`.
// loc_mask bit d set => Vertex along d. Returns CG_OK or records CG_ERR_ARG.
int cg_check_field(cg_ctx* ctx, const cg_grid* grid, const cg_field& f, int dtype, int loc_mask,
                   const char* name);
int cg_check_grid(cg_ctx* ctx, const cg_grid* grid);

inline bool cg_present(const cg_field& f) { return f.data != nullptr; }

// Run `capture(stream)` into a CUDA graph cached under `key` and launch it.
template <class F>
int cg_graph_run(cg_ctx* ctx, const std::string& key, F&& capture);

// ---- small helpers -------------------------------------------------------------------------
inline int cg_div_up(long a, long b) { return (int)((a + b - 1) / b); }

template <class F>
int cg_graph_run(cg_ctx* ctx, const std::string& key, F&& capture) {
    cg_graph_entry* hit = nullptr;
    for (auto& g : ctx->graphs)
        if (g.exec && g.key == key) hit = &g;
    if (!hit) {
        cg_graph_entry& slot = ctx->graphs[ctx->graph_next];
        ctx->graph_next = (ctx->graph_next + 1) % 8;
        if (slot.exec) {
            cudaGraphExecDestroy(slot.exec);
            slot.exec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        CG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int rc = capture(ctx->stream);
        cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
        if (rc != CG_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess) return cg_fail(ctx, CG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
        cudaError_t ie = cudaGraphInstantiate(&slot.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            slot.exec = nullptr;
            return cg_fail(ctx, CG_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ie));
        }
        slot.key = key;
        hit = &slot;
    }
    CG_CUDA(ctx, cudaGraphLaunch(hit->exec, ctx->stream));
    return CG_OK;
}

// Append the raw bytes of a POD value to a graph key.
template <class V>
inline void cg_key_add(std::string& k, const V& v) {
    k.append(reinterpret_cast<const char*>(&v), sizeof(V));
}
