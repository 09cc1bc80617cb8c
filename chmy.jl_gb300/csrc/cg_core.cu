// cg_core.cu — context, memory, argument checks, the fused boundary-condition kernel and the
// max-norm reduction of libchmy_gb300.
#include <cstdarg>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include "cg_common.cuh"

// Message of the calling thread's last failure in a call without a context (cg_init,
// cg_maxabs_noalloc, ...): one buffer per host thread, so concurrent callers never garble
// each other's text.
static thread_local char g_init_err[512] = "";

int cg_fail(cg_ctx* ctx, int code, const char* fmt, ...) {
    char* dst = ctx ? ctx->err : g_init_err;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(dst, 512, fmt, ap);
    va_end(ap);
    return code;
}

extern "C" int cg_abi_version(void) { return CG_ABI_VERSION; }

extern "C" const char* cg_last_error(const cg_ctx* ctx) { return ctx ? ctx->err : g_init_err; }

extern "C" int cg_init(int device, cg_ctx** out) {
    if (!out) return cg_fail(nullptr, CG_ERR_ARG, "cg_init: out is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return cg_fail(nullptr, CG_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
    if (device < 0 || device >= ndev)
        return cg_fail(nullptr, CG_ERR_ARG, "cg_init: device %d not in [0, %d)", device, ndev);
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return cg_fail(nullptr, CG_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    cg_ctx* ctx = new cg_ctx();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    // a blocking stream: ordered with work on the legacy default stream (e.g. host-side
    // copies issued by PyTorch or CUDA.jl) without extra synchronisation
    e = cudaStreamCreate(&ctx->own_stream);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_red, sizeof(unsigned long long) * cg_ctx::kRedSlots);
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_red, sizeof(unsigned long long) * cg_ctx::kRedSlots);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e != cudaSuccess) {
        cg_fail(nullptr, CG_ERR_CUDA, "cg_init: %s", cudaGetErrorString(e));
        cg_destroy(ctx);
        return CG_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
    return CG_OK;
}

extern "C" int cg_destroy(cg_ctx* ctx) {
    if (!ctx) return CG_OK;
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    for (auto& g : ctx->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (ctx->dc_pool) cudaFree(ctx->dc_pool);
    for (int s = 0; s < cg_ctx::kScratchSlots; ++s)
        if (ctx->scratch[s]) cudaFree(ctx->scratch[s]);
    if (ctx->d_red) cudaFree(ctx->d_red);
    if (ctx->h_red) cudaFreeHost(ctx->h_red);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return CG_OK;
}

namespace {
std::mutex g_tune_mu;
std::map<std::string, cg_tune_cfg> g_tune;
}  // namespace

bool cg_autotune_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("CG_AUTOTUNE");
        return !(e && e[0] == '0');
    }();
    return on;
}

bool cg_tune_forced(cg_tune_cfg* out) {
    // CG_MARCH_LAYOUT=<segment length>:<variant> fixes the march kernels' launch layout (0 as
    // the segment length keeps the launcher's rule; variant: in 3D 0-1 the register-fed block
    // shapes and 2-3 the TMA-fed ones, in 2D 1 and 2 for two iterations per pass): for
    // profiling one layout without timing the candidates first
    const char* e = std::getenv("CG_MARCH_LAYOUT");
    if (!e || !e[0]) return false;
    int seg = 0, var = 0;
    if (std::sscanf(e, "%d:%d", &seg, &var) != 2 || seg < 0 || var < 0 || var > 3) return false;
    *out = cg_tune_cfg{seg, var};
    return true;
}

bool cg_block_forced(dim3* out) {
    const char* e = std::getenv("CG_BLOCK");
    if (!e || !e[0]) return false;
    int bx = 0, by = 0;
    if (std::sscanf(e, "%dx%d", &bx, &by) != 2) return false;
    if (bx < 32 || bx % 32 || by < 1 || bx * by < 64 || bx * by > 1024) return false;
    *out = dim3((unsigned)bx, (unsigned)by);
    return true;
}

bool cg_pdl_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("CG_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

bool cg_bc_fold_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("CG_BC_FOLD");
        return !(e && e[0] == '0');
    }();
    return on;
}

bool cg_ptdiff_fused_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("CG_PTDIFF_FUSED");
        return !(e && e[0] == '0');
    }();
    return on;
}

bool cg_sia_persistent_enabled() {
    // read on every call (once per run), so that a process can compare both forms
    const char* e = std::getenv("CG_SIA_PERSISTENT");
    return e && e[0] == '1';
}

int cg_sia_tile_rows_forced() {
    // read on every call, like CG_SIA_PERSISTENT
    const char* e = std::getenv("CG_SIA_TILE_ROWS");
    if (!e) return 0;
    const long r = std::strtol(e, nullptr, 10);
    return (r == 4 || r == 8 || r == 16) ? (int)r : 0;
}

cg_barrier_cfg cg_sia_barrier_cfg() {
    // read on every call, like CG_SIA_PERSISTENT
    cg_barrier_cfg c;
    if (const char* e = std::getenv("CG_SIA_BARRIER_LIMIT_MS")) {
        const long ms = std::strtol(e, nullptr, 10);
        if (ms >= 1 && ms <= 60000) c.limit_ns = (unsigned long long)ms * 1000000ull;
    }
    if (const char* e = std::getenv("CG_SIA_BARRIER_WITHHELD")) {
        const long w = std::strtol(e, nullptr, 10);
        if (w >= 0 && w <= 1024) c.withheld = (int)w;
    }
    return c;
}

cg_tma_cfg cg_tma_wait_cfg() {
    cg_tma_cfg c;
    if (const char* e = std::getenv("CG_TMA_WAIT_LIMIT_MS")) {
        const long ms = std::strtol(e, nullptr, 10);
        if (ms >= 1 && ms <= 60000) c.limit_ns = (unsigned long long)ms * 1000000ull;
    }
    if (const char* e = std::getenv("CG_TMA_WITHHOLD_PLANE")) {
        const long m = std::strtol(e, nullptr, 10);
        if (m >= 0 && m <= 1000000) c.withhold = (int)m;
    }
    return c;
}

bool cg_tune_verbose() {
    static const bool on = [] {
        const char* e = std::getenv("CG_TUNE_VERBOSE");
        return e && e[0] == '1';
    }();
    return on;
}

bool cg_tune_lookup(const std::string& key, cg_tune_cfg* out) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it == g_tune.end()) return false;
    *out = it->second;
    return true;
}

void cg_tune_store(const std::string& key, const cg_tune_cfg& cfg) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = cfg;
}

int* cg_tma_flag(cg_ctx* ctx, int* rc) {
    int* e = static_cast<int*>(cg_scratch(ctx, 10, 256, rc));
    if (*rc) return nullptr;
    if (cudaMemsetAsync(e, 0, sizeof(int), ctx->stream) != cudaSuccess) {
        *rc = cg_fail(ctx, CG_ERR_CUDA, "clearing the TMA wait flag failed");
        return nullptr;
    }
    return e;
}

int cg_tma_check(cg_ctx* ctx, int* flag, const char* what) {
    int h = 0;
    CG_CUDA(ctx, cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h) return cg_fail(ctx, CG_ERR_TIMEOUT, "%s: a wait for staged data timed out", what);
    return CG_OK;
}

void* cg_scratch(cg_ctx* ctx, int slot, size_t bytes, int* rc) {
    *rc = CG_OK;
    if (slot < 0 || slot >= cg_ctx::kScratchSlots) {
        *rc = cg_fail(ctx, CG_ERR_ARG, "scratch slot %d out of range", slot);
        return nullptr;
    }
    if (ctx->scratch_bytes[slot] >= bytes) return ctx->scratch[slot];
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess && ctx->scratch[slot]) e = cudaFree(ctx->scratch[slot]);
    ctx->scratch[slot] = nullptr;
    ctx->scratch_bytes[slot] = 0;
    if (e == cudaSuccess) e = cudaMalloc(&ctx->scratch[slot], bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->scratch[slot], 0, bytes, ctx->stream);
    if (e != cudaSuccess) {
        ctx->scratch[slot] = nullptr;
        *rc = cg_fail(ctx, CG_ERR_CUDA, "scratch allocation of %zu bytes: %s", bytes, cudaGetErrorString(e));
        return nullptr;
    }
    ctx->scratch_bytes[slot] = bytes;
    return ctx->scratch[slot];
}

extern "C" int cg_set_stream(cg_ctx* ctx, void* stream) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_set_stream: ctx is NULL");
    ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    return CG_OK;
}

extern "C" int cg_sync(cg_ctx* ctx) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_sync: ctx is NULL");
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CG_OK;
}

// ---- argument checks -----------------------------------------------------------------------

int cg_check_grid(cg_ctx* ctx, const cg_grid* grid) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "ctx is NULL");
    if (!grid) return cg_fail(ctx, CG_ERR_ARG, "grid is NULL");
    if (grid->ndim < 1 || grid->ndim > 3) return cg_fail(ctx, CG_ERR_ARG, "grid ndim %d not in 1..3", grid->ndim);
    for (int d = 0; d < grid->ndim; ++d)
        if (grid->n[d] < 2) return cg_fail(ctx, CG_ERR_ARG, "grid n[%d] = %d < 2", d, grid->n[d]);
    return CG_OK;
}

int cg_check_field(cg_ctx* ctx, const cg_grid* grid, const cg_field& f, int dtype, int loc_mask, const char* name) {
    if (!f.data) return cg_fail(ctx, CG_ERR_ARG, "%s: data is NULL", name);
    if (f.dtype != dtype) return cg_fail(ctx, CG_ERR_ARG, "%s: dtype %d, expected %d", name, f.dtype, dtype);
    if (f.ndim != grid->ndim) return cg_fail(ctx, CG_ERR_ARG, "%s: ndim %d, grid has %d", name, f.ndim, grid->ndim);
    for (int d = 0; d < f.ndim; ++d) {
        const int want_loc = (loc_mask >> d) & 1;
        if (loc_mask >= 0 && f.loc[d] != want_loc)
            return cg_fail(ctx, CG_ERR_ARG, "%s: location along dim %d is %s, expected %s", name, d,
                           f.loc[d] ? "Vertex" : "Center", want_loc ? "Vertex" : "Center");
        if (f.n[d] != grid->n[d] + f.loc[d])
            return cg_fail(ctx, CG_ERR_ARG, "%s: extent n[%d] = %d does not match grid (%d)", name, d, f.n[d],
                           grid->n[d] + f.loc[d]);
        if (f.halo[d] < 1) return cg_fail(ctx, CG_ERR_ARG, "%s: halo[%d] = %d < 1", name, d, f.halo[d]);
    }
    if (f.stride[0] != 1) return cg_fail(ctx, CG_ERR_ARG, "%s: stride[0] must be 1", name);
    if (f.ndim > 1 && f.stride[1] < f.n[0] + 4 * f.halo[0])
        return cg_fail(ctx, CG_ERR_ARG, "%s: stride[1] smaller than the padded x extent", name);
    if (f.ndim > 2 && f.stride[2] < f.stride[1] * (f.n[1] + 4 * f.halo[1]))
        return cg_fail(ctx, CG_ERR_ARG, "%s: stride[2] smaller than the padded xy plane", name);
    return CG_OK;
}

// ---- memory ----------------------------------------------------------------------------------

extern "C" int cg_field_alloc(cg_ctx* ctx, int dtype, int ndim, const int32_t n[3], const int32_t loc[3],
                              const int32_t halo[3], int pitch_align, cg_field* out) {
    if (!ctx || !out || !n || !loc || !halo) return cg_fail(ctx, CG_ERR_ARG, "cg_field_alloc: NULL argument");
    if (dtype != CG_F32 && dtype != CG_F64) return cg_fail(ctx, CG_ERR_ARG, "cg_field_alloc: bad dtype %d", dtype);
    if (ndim < 1 || ndim > 3) return cg_fail(ctx, CG_ERR_ARG, "cg_field_alloc: bad ndim %d", ndim);
    if (pitch_align && (pitch_align < 16 || (pitch_align & (pitch_align - 1))))
        return cg_fail(ctx, CG_ERR_ARG, "cg_field_alloc: pitch_align %d is not a power of two >= 16", pitch_align);
    const int esz = dtype == CG_F64 ? 8 : 4;
    cg_field f;
    std::memset(&f, 0, sizeof(f));
    f.dtype = dtype;
    f.ndim = ndim;
    long ext[3] = {1, 1, 1};
    for (int d = 0; d < 3; ++d) {
        if (d < ndim) {
            if (n[d] < 1 || halo[d] < 0 || (loc[d] != 0 && loc[d] != 1))
                return cg_fail(ctx, CG_ERR_ARG, "cg_field_alloc: bad extent/halo/location along dim %d", d);
            f.n[d] = n[d];
            f.loc[d] = loc[d];
            f.halo[d] = halo[d];
            ext[d] = n[d] + 4L * halo[d];
        } else {
            f.n[d] = 1;
        }
    }
    long front = 0, pitch = ext[0];
    if (pitch_align) {
        const long a = pitch_align / esz;
        front = (a - (2L * f.halo[0] - 1) % a) % a;
        pitch = ((front + ext[0] + a - 1) / a) * a;
    }
    f.stride[0] = 1;
    f.stride[1] = ndim > 1 ? pitch : 0;
    f.stride[2] = ndim > 2 ? pitch * ext[1] : 0;
    const size_t count = (size_t)pitch * ext[1] * ext[2] + (size_t)front;
    void* base = nullptr;
    CG_CUDA(ctx, cudaMalloc(&base, count * esz));
    CG_CUDA(ctx, cudaMemsetAsync(base, 0, count * esz, ctx->stream));
    f.data = static_cast<char*>(base) + front * esz;
    f.pad_ = (int32_t)front;
    *out = f;
    return CG_OK;
}

extern "C" int cg_field_free(cg_ctx* ctx, cg_field* f) {
    if (!ctx || !f) return cg_fail(ctx, CG_ERR_ARG, "cg_field_free: NULL argument");
    if (!f->data) return CG_OK;
    const int esz = f->dtype == CG_F64 ? 8 : 4;
    void* base = static_cast<char*>(f->data) - (long)f->pad_ * esz;
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    CG_CUDA(ctx, cudaFree(base));
    f->data = nullptr;
    return CG_OK;
}

static int field_copy(cg_ctx* ctx, const cg_field* f, void* host, bool up) {
    if (!ctx || !f || !f->data || !host) return cg_fail(ctx, CG_ERR_ARG, "field copy: NULL argument");
    const int esz = f->dtype == CG_F64 ? 8 : 4;
    long ext[3] = {1, 1, 1};
    for (int d = 0; d < f->ndim; ++d) ext[d] = f->n[d] + 4L * f->halo[d];
    const size_t row = (size_t)ext[0] * esz;
    const size_t dpitch = f->ndim > 1 ? (size_t)f->stride[1] * esz : row;
    const size_t plane = f->ndim > 2 ? (size_t)f->stride[2] * esz : dpitch * ext[1];
    const bool dense_planes = (plane == dpitch * ext[1]);
    cudaMemcpyKind kind = up ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
    if (dense_planes) {
        if (up)
            CG_CUDA(ctx, cudaMemcpy2DAsync(f->data, dpitch, host, row, row, ext[1] * ext[2], kind, ctx->stream));
        else
            CG_CUDA(ctx, cudaMemcpy2DAsync(host, row, f->data, dpitch, row, ext[1] * ext[2], kind, ctx->stream));
    } else {
        for (long k = 0; k < ext[2]; ++k) {
            char* dev = static_cast<char*>(f->data) + k * plane;
            char* hst = static_cast<char*>(host) + k * row * ext[1];
            if (up)
                CG_CUDA(ctx, cudaMemcpy2DAsync(dev, dpitch, hst, row, row, ext[1], kind, ctx->stream));
            else
                CG_CUDA(ctx, cudaMemcpy2DAsync(hst, row, dev, dpitch, row, ext[1], kind, ctx->stream));
        }
    }
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CG_OK;
}

extern "C" int cg_field_upload(cg_ctx* ctx, const cg_field* f, const void* host_dense) {
    return field_copy(ctx, f, const_cast<void*>(host_dense), true);
}
extern "C" int cg_field_download(cg_ctx* ctx, const cg_field* f, void* host_dense) {
    return field_copy(ctx, f, host_dense, false);
}

// ---- boundary conditions: one launch per batch ------------------------------------------------
//
// Chmy applies a batch as 2N launches, Dim N -> 1 and Side(1) then Side(2), each over the
// tangential indices 0..n+2 (src/BoundaryConditions/batch.jl:104-113,243-268); a phase
// reads the value one step inward, so a later phase can read what an earlier one wrote
// (edges and corners). Here every written point is handled by exactly one thread — the
// one of its LAST writing phase — which evaluates the chain of ghost rules back to a
// point no phase writes (or to a Dirichlet constant). Points no phase writes are never
// modified during the launch, so the single launch has no read/write race.

namespace {

constexpr int kBcMaxFields = 8;
constexpr int kBcMaxItems = kBcMaxFields * 12;

template <class T>
struct BcField {
    T* p;          // logical index 0
    long s[3];
    int ext[3];    // field extent per dim
    int loc[3];
    int kind[3][2];
    T val[3][2];
    const T* va[3][2];  // per-point values over the tangential indices 0..n_t+2, or NULL
    T h[3];
};

// BoundaryFunction sides of a batch (cg_bc_fn), a separate kernel argument of the launches that
// have some: per field, dimension and side the function, its evaluation location (Vertex 1,
// Center 0, the same for every dimension) and whether the coordinate along the condition's
// dimension is an argument; and the grid's coordinates.
template <class T, bool FN>
struct BcFns {};
template <class T>
struct BcFns<T, true> {
    cgk::FnDev<T> fn[kBcMaxFields][3][2];
    unsigned char vtx[kBcMaxFields][3][2];
    unsigned char full[kBcMaxFields][3][2];
    T org[3], dx[3];
};

// The value of phase (d, s) of field fi at the point q: its BoundaryFunction at q's coordinates,
// else the per-point array at q's tangential indices (remove_dim(dim, I)), else the constant.
template <class T, bool FN>
__device__ __forceinline__ T bc_value(const BcField<T>& F, const BcFns<T, FN>& fns, int fi, int nd, const int* n, int d,
                                      int s, const int* q) {
    if constexpr (FN) {
        const cgk::FnDev<T>& fn = fns.fn[fi][d][s];
        if (fn.kind != CG_FN_NONE) {
            T x[3] = {T(0), T(0), T(0)};
            int m = 0;
            for (int t = 0; t < nd; ++t) {
                if (t == d && !fns.full[fi][d][s]) continue;
                x[m++] = cgk::grid_coord(fns.org[t], fns.dx[t], q[t], fns.vtx[fi][d][s] != 0);
            }
            return cgk::fn_eval(fn, m, x);
        }
    }
    const T* a = F.va[d][s];
    if (!a) return F.val[d][s];
    long idx = 0, mul = 1;
    for (int t = 0; t < nd; ++t) {
        if (t == d) continue;
        idx += (long)q[t] * mul;
        mul *= n[t] + 3;
    }
    return a[idx];
}

// One boundary plane of one field. lo/hi: the tangential indices (the lower tangential
// dimension first) that lie on no phase plane of their dimension; a point inside both ranges is
// written by this phase alone, from the interior source `src` (rule `rule`) that no earlier
// phase writes, so the kernel takes it without walking the phase chain (lo > hi: never).
struct BcItem {
    int field, d, s, plane, start;
    int src, rule;
    int lo[2], hi[2];
};

template <class T>
struct BcBatch {
    int nd;
    int n[3];
    int nitems;
    int total;
    BcField<T> f[kBcMaxFields];
    BcItem items[kBcMaxItems];
};

enum { R_CONST = 0, R_DIR_C = 1, R_NEU = 2, R_COPY = 3 };

// Planes written by phase (d, s): ghost index g, source index src and rule.
template <class T>
__host__ __device__ inline int phase_planes(const BcField<T>& F, const int* n, int d, int s, int* g, int* src,
                                            int* rule) {
    const int kind = F.kind[d][s];
    const int ext = F.ext[d];
    const bool vtx = F.loc[d] == CG_VERTEX;
    switch (kind) {
        case CG_BC_DIRICHLET:
            if (vtx) {
                g[0] = s ? ext : 1;
                src[0] = -1;
                rule[0] = R_CONST;
            } else {
                g[0] = s ? ext + 1 : 0;
                src[0] = s ? ext : 1;
                rule[0] = R_DIR_C;
            }
            return 1;
        case CG_BC_NEUMANN:
            g[0] = s ? ext + 1 : 0;
            src[0] = s ? ext : 1;
            rule[0] = R_NEU;
            return 1;
        case CG_BC_PERIODIC:
            if (s == 0) {
                g[0] = 0;
                src[0] = n[d];
                rule[0] = R_COPY;
                return 1;
            }
            g[0] = n[d] + 1;
            src[0] = 1;
            rule[0] = R_COPY;
            if (vtx) {
                g[1] = n[d] + 2;
                src[1] = 2;
                rule[1] = R_COPY;
                return 2;
            }
            return 1;
        default:
            return 0;
    }
}

// Phase order index k <-> (d, s): k = (nd-1-d)*2 + s.
template <class T>
__device__ inline bool phase_member(const BcField<T>& F, int nd, const int* n, int k, const int* p, int* src,
                                    int* rule) {
    const int d = nd - 1 - (k >> 1), s = k & 1;
    for (int t = 0; t < nd; ++t)
        if (t != d && (p[t] < 0 || p[t] > n[t] + 2)) return false;
    int g[2], sr[2], ru[2];
    const int np = phase_planes(F, n, d, s, g, sr, ru);
    for (int q = 0; q < np; ++q)
        if (p[d] == g[q]) {
            *src = sr[q];
            *rule = ru[q];
            return true;
        }
    return false;
}

// One thread per point of one item (a boundary plane of one field): blockIdx.z is the item, x
// and y the plane's tangential indices (the lower dimension along x). The dimension count is a
// template parameter, so the phase loops unroll with the phase, dimension and side known at
// compile time and the rule chain stays in registers.
template <class T, bool FN, int ND>
__global__ void bc_apply_kernel(const BcBatch<T> b, const BcFns<T, FN> fns) {
    cg_dep_wait();
    cg_dep_release();
    const BcItem item = b.items[blockIdx.z];
    const int dd = item.d;
    const int ia = blockIdx.x * blockDim.x + threadIdx.x, ib = blockIdx.y * blockDim.y + threadIdx.y;
    // the point: tangential indices 0..n_t+2, the item's plane along dd
    int p[3] = {0, 0, 0};
    if constexpr (ND == 1) {
        if (ia > 0 || ib > 0) return;
        p[0] = item.plane;
    } else if constexpr (ND == 2) {
        const int ta = dd == 0 ? 1 : 0;
        if (ia > b.n[ta] + 2 || ib > 0) return;
        p[0] = dd == 0 ? item.plane : ia;
        p[1] = dd == 1 ? item.plane : ia;
    } else {
        const int ta = dd == 0 ? 1 : 0, tb = dd == 2 ? 1 : 2;
        if (ia > b.n[ta] + 2 || ib > b.n[tb] + 2) return;
        p[0] = dd == 0 ? item.plane : ia;
        p[1] = dd == 1 ? item.plane : (dd == 0 ? ia : ib);
        p[2] = dd == 2 ? item.plane : ib;
    }
    const BcField<T>& F = b.f[item.field];
    if (ia >= item.lo[0] && ia <= item.hi[0] && (ND < 3 || (ib >= item.lo[1] && ib <= item.hi[1]))) {
        // on no other phase's plane: this phase's rule on its source, as the chain walk below
        // takes it for such a point
        const T v = bc_value(F, fns, item.field, ND, b.n, dd, item.s, p);
        T base = v;
        if (item.rule != R_CONST) {
            int q[3] = {p[0], p[1], p[2]};
            q[dd] = item.src;
            base = F.p[q[0] + q[1] * F.s[1] + q[2] * F.s[2]];
            if (item.rule == R_DIR_C) base = fma(T(2), v - base, base);
            else if (item.rule == R_NEU) base = fma(F.h[dd], item.s == 0 ? -v : v, base);
        }
        F.p[p[0] + p[1] * F.s[1] + p[2] * F.s[2]] = base;
        return;
    }
    const int k0 = (ND - 1 - dd) * 2 + item.s;
    int src, rule;
    // only the last writing phase handles the point
#pragma unroll
    for (int k = 0; k < 2 * ND; ++k)
        if (k > k0 && phase_member(F, ND, b.n, k, p, &src, &rule)) return;
    // walk the chain of rules back from phase k0 to an unwritten point or a constant: at most
    // one rule per phase, in decreasing phase order (the largest earlier phase that writes the
    // current point next)
    int q[3] = {p[0], p[1], p[2]};
    bool used[2 * ND];
    int rk[2 * ND];
    T vk[2 * ND];
    bool open = true;
    T base = T(0);
#pragma unroll
    for (int k = 2 * ND - 1; k >= 0; --k) {
        used[k] = false;
        rk[k] = R_CONST;
        vk[k] = T(0);
        if (!open || k > k0 || !phase_member(F, ND, b.n, k, q, &src, &rule)) continue;
        const int d = ND - 1 - (k >> 1), s = k & 1;
        const T v = bc_value(F, fns, item.field, ND, b.n, d, s, q);
        if (rule == R_CONST) {
            base = v;
            open = false;
            continue;
        }
        used[k] = true;
        rk[k] = rule;
        vk[k] = v;
        q[d] = src;
    }
    if (open) base = F.p[q[0] + q[1] * F.s[1] + q[2] * F.s[2]];
    // apply the rules from the innermost (lowest phase) out
#pragma unroll
    for (int k = 0; k < 2 * ND; ++k) {
        if (!used[k]) continue;
        const int d = ND - 1 - (k >> 1), s = k & 1;
        switch (rk[k]) {
            case R_DIR_C: base = fma(T(2), vk[k] - base, base); break;
            case R_NEU: base = fma(F.h[d], s == 0 ? -vk[k] : vk[k], base); break;
            default: break;
        }
    }
    F.p[p[0] + p[1] * F.s[1] + p[2] * F.s[2]] = base;
}

// Launch of bc_apply_kernel over the batch's items: blocks of 32 x 8 points (3D), 128 (2D) or one
// thread (1D), the grid covering the largest tangential extents of the items.
template <class T, bool FN>
cudaError_t bc_launch(const BcBatch<T>& b, const BcFns<T, FN>& fns, cudaStream_t st, bool dep) {
    int ea = 1, eb = 1;
    for (int i = 0; i < b.nitems; ++i) {
        const int d = b.items[i].d;
        if (b.nd >= 2) ea = std::max(ea, b.n[d == 0 ? 1 : 0] + 3);
        if (b.nd == 3) eb = std::max(eb, b.n[d == 2 ? 1 : 2] + 3);
    }
    const unsigned nz = (unsigned)b.nitems;
    if (b.nd == 3)
        return cg_launch(bc_apply_kernel<T, FN, 3>, dim3(cg_div_up(ea, 32), cg_div_up(eb, 8), nz), dim3(32, 8), 0, st, dep,
                         b, fns);
    if (b.nd == 2)
        return cg_launch(bc_apply_kernel<T, FN, 2>, dim3(cg_div_up(ea, 128), 1, nz), dim3(128), 0, st, dep, b, fns);
    return cg_launch(bc_apply_kernel<T, FN, 1>, dim3(1, 1, nz), dim3(32), 0, st, dep, b, fns);
}

// The item's fast-path ranges (BcItem::lo/hi): per tangential dimension t, the indices between
// its lower and its upper phase planes. Empty (every point takes the chain walk) when the other
// side of the item's own dimension shares its plane (tiny grids) or, for the upper side, holds
// its source.
template <class T>
void bc_fast_ranges(const BcField<T>& F, int nd, const int* n, int d, int s, int plane, int src, int rule, BcItem* it) {
    {
        int g[2], sr[2], ru[2];
        const int np = phase_planes(F, n, d, 1 - s, g, sr, ru);
        for (int q = 0; q < np; ++q)
            if (g[q] == plane || (s == 1 && rule != R_CONST && g[q] == src)) return;  // lo > hi: no fast path
    }
    int m = 0;
    for (int t = 0; t < nd; ++t) {
        if (t == d) continue;
        int lo = 0, hi = n[t] + 2;
        const int mid = (n[t] + 2) / 2;
        for (int ss = 0; ss < 2; ++ss) {
            int g[2], sr[2], ru[2];
            const int np = phase_planes(F, n, t, ss, g, sr, ru);
            for (int q = 0; q < np; ++q) {
                if (g[q] <= mid) lo = std::max(lo, g[q] + 1);
                else hi = std::min(hi, g[q] - 1);
            }
        }
        it->lo[m] = lo;
        it->hi[m] = hi;
        ++m;
    }
    for (; m < 2; ++m) {  // dimensions the grid does not have: index 0 only
        it->lo[m] = 0;
        it->hi[m] = 0;
    }
}

template <class T>
int bc_apply_t(cg_ctx* ctx, const cg_grid* grid, int nfields, const cg_field* fields, const cg_bc* bcs, bool dep,
               const cg_bc_fn* fns = nullptr) {
    BcBatch<T> b;
    std::memset(&b, 0, sizeof(b));
    b.nd = grid->ndim;
    for (int d = 0; d < 3; ++d) b.n[d] = d < b.nd ? grid->n[d] : 1;
    int total = 0, ni = 0;
    for (int fi = 0; fi < nfields; ++fi) {
        const cg_field& f = fields[fi];
        BcField<T>& F = b.f[fi];
        F.p = static_cast<T*>(f.data) + cg_origin_offset(f);
        for (int d = 0; d < 3; ++d) {
            F.s[d] = d < f.ndim ? (long)f.stride[d] : 0;
            F.ext[d] = d < f.ndim ? f.n[d] : 1;
            F.loc[d] = d < f.ndim ? f.loc[d] : 0;
            F.h[d] = (T)grid->spacing[d];
            for (int s = 0; s < 2; ++s) {
                F.kind[d][s] = d < f.ndim ? bcs[fi].kind[d][s] : CG_BC_NONE;
                F.val[d][s] = (T)bcs[fi].value[d][s];
                F.va[d][s] = d < f.ndim ? static_cast<const T*>(bcs[fi].values[d][s]) : nullptr;
            }
        }
        for (int d = 0; d < b.nd; ++d) {
            const bool p0 = F.kind[d][0] == CG_BC_PERIODIC, p1 = F.kind[d][1] == CG_BC_PERIODIC;
            if (p0 != p1) return cg_fail(ctx, CG_ERR_ARG, "bc: periodic must be set on both sides of dim %d", d);
        }
        for (int d = b.nd - 1; d >= 0; --d)
            for (int s = 0; s < 2; ++s) {
                int g[2], src[2], rule[2];
                const int np = phase_planes(F, b.n, d, s, g, src, rule);
                long cnt = 1;
                for (int t = 0; t < b.nd; ++t)
                    if (t != d) cnt *= (b.n[t] + 3);
                for (int q = 0; q < np; ++q) {
                    if (ni >= kBcMaxItems) return cg_fail(ctx, CG_ERR_ARG, "bc: too many boundary planes");
                    BcItem it{fi, d, s, g[q], total, src[q], rule[q], {0, 0}, {-1, -1}};
                    bc_fast_ranges(F, b.nd, b.n, d, s, g[q], src[q], rule[q], &it);
                    b.items[ni] = it;
                    ++ni;
                    total += (int)cnt;
                }
            }
    }
    b.nitems = ni;
    b.total = total;
    if (total == 0) return CG_OK;
    bool any_fn = false;
    if (fns)
        for (int fi = 0; fi < nfields; ++fi)
            for (int d = 0; d < b.nd; ++d)
                for (int s = 0; s < 2; ++s) any_fn = any_fn || fns[fi].fn[d][s].kind != CG_FN_NONE;
    if (!any_fn) {
        CG_CUDA(ctx, bc_launch(b, BcFns<T, false>{}, ctx->stream, dep));
        return CG_OK;
    }
    BcFns<T, true> bf;
    std::memset(&bf, 0, sizeof(bf));
    for (int d = 0; d < 3; ++d) {
        bf.org[d] = (T)grid->origin[d];
        bf.dx[d] = (T)grid->spacing[d];
    }
    for (int fi = 0; fi < nfields; ++fi)
        for (int d = 0; d < b.nd; ++d)
            for (int s = 0; s < 2; ++s) {
                const cg_function& fn = fns[fi].fn[d][s];
                if (fn.kind == CG_FN_NONE) continue;
                const int kind = b.f[fi].kind[d][s];
                bf.fn[fi][d][s].kind = fn.kind;
                for (int q = 0; q < 8; ++q) bf.fn[fi][d][s].p[q] = (T)fn.p[q];
                // Dirichlet: the field's location along d; Neumann: its flip
                const bool vtx = b.f[fi].loc[d] == CG_VERTEX;
                bf.vtx[fi][d][s] = (unsigned char)(kind == CG_BC_NEUMANN ? !vtx : vtx);
                bf.full[fi][d][s] = (unsigned char)(fns[fi].full_dims[d][s] != 0);
            }
    CG_CUDA(ctx, bc_launch(b, bf, ctx->stream, dep));
    return CG_OK;
}

// The function sides of a batch: known forms, on Dirichlet or Neumann sides only.
int check_bc_fns(cg_ctx* ctx, const cg_grid* grid, int nfields, const cg_bc* bcs, const cg_bc_fn* fns) {
    for (int fi = 0; fi < nfields; ++fi)
        for (int d = 0; d < 3; ++d)
            for (int s = 0; s < 2; ++s) {
                const int k = fns[fi].fn[d][s].kind;
                if (k == CG_FN_NONE) continue;
                if (k < CG_FN_CONST || k > CG_FN_AFFINE)
                    return cg_fail(ctx, CG_ERR_ARG, "cg_bc_apply_fn: field %d dim %d side %d: unknown function kind %d", fi,
                                   d, s, k);
                if (d >= grid->ndim)
                    return cg_fail(ctx, CG_ERR_ARG, "cg_bc_apply_fn: a function on dim %d of a %dD grid", d, grid->ndim);
                const int kind = bcs[fi].kind[d][s];
                if (kind != CG_BC_DIRICHLET && kind != CG_BC_NEUMANN)
                    return cg_fail(ctx, CG_ERR_ARG,
                                   "cg_bc_apply_fn: field %d dim %d side %d: a function needs a Dirichlet or Neumann side",
                                   fi, d, s);
            }
    return CG_OK;
}

}  // namespace

int cg_bc_apply_impl(cg_ctx* ctx, const cg_grid* grid, int nfields, const cg_field* fields, const cg_bc* bcs, bool dep) {
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (nfields < 0 || nfields > kBcMaxFields)
        return cg_fail(ctx, CG_ERR_ARG, "cg_bc_apply: nfields %d not in 0..%d", nfields, kBcMaxFields);
    if (nfields == 0) return CG_OK;
    if (!fields || !bcs) return cg_fail(ctx, CG_ERR_ARG, "cg_bc_apply: NULL fields or bcs");
    if (grid->ndim >= 2)
        for (int d = 0; d < grid->ndim; ++d)
            if (grid->n[d] < 2) return cg_fail(ctx, CG_ERR_ARG, "cg_bc_apply: grid too small");
    const int dtype = fields[0].dtype;
    for (int i = 0; i < nfields; ++i) {
        rc = cg_check_field(ctx, grid, fields[i], dtype, -1, "cg_bc_apply field");
        if (rc) return rc;
    }
    return dtype == CG_F64 ? bc_apply_t<double>(ctx, grid, nfields, fields, bcs, dep)
                           : bc_apply_t<float>(ctx, grid, nfields, fields, bcs, dep);
}

extern "C" int cg_bc_apply(cg_ctx* ctx, const cg_grid* grid, int nfields, const cg_field* fields, const cg_bc* bcs) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_bc_apply: ctx is NULL");
    cudaSetDevice(ctx->device);
    return cg_bc_apply_impl(ctx, grid, nfields, fields, bcs);
}

extern "C" int cg_bc_apply_fn(cg_ctx* ctx, const cg_grid* grid, int nfields, const cg_field* fields, const cg_bc* bcs,
                              const cg_bc_fn* fns) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_bc_apply_fn: ctx is NULL");
    if (!fns) return cg_bc_apply(ctx, grid, nfields, fields, bcs);
    int rc = cg_check_grid(ctx, grid);
    if (rc) return rc;
    if (nfields < 0 || nfields > kBcMaxFields)
        return cg_fail(ctx, CG_ERR_ARG, "cg_bc_apply_fn: nfields %d not in 0..%d", nfields, kBcMaxFields);
    if (nfields == 0) return CG_OK;
    if (!fields || !bcs) return cg_fail(ctx, CG_ERR_ARG, "cg_bc_apply_fn: NULL fields or bcs");
    if ((rc = check_bc_fns(ctx, grid, nfields, bcs, fns))) return rc;
    if (grid->ndim >= 2)
        for (int d = 0; d < grid->ndim; ++d)
            if (grid->n[d] < 2) return cg_fail(ctx, CG_ERR_ARG, "cg_bc_apply_fn: grid too small");
    const int dtype = fields[0].dtype;
    for (int i = 0; i < nfields; ++i)
        if ((rc = cg_check_field(ctx, grid, fields[i], dtype, -1, "cg_bc_apply_fn field"))) return rc;
    cudaSetDevice(ctx->device);
    return dtype == CG_F64 ? bc_apply_t<double>(ctx, grid, nfields, fields, bcs, false, fns)
                           : bc_apply_t<float>(ctx, grid, nfields, fields, bcs, false, fns);
}

// ---- max-norm over interiors: one launch for up to kRedSlots fields --------------------------

namespace {

constexpr int kMaxRedFields = 16;

struct RedField {
    const void* p;  // logical index (1,1,1)
    long s1, s2;
    int n0, n1, n2;
    int is64;
};
struct RedBatch {
    int nfields;
    RedField f[kMaxRedFields];
};

__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ unsigned long long abs_bits(float v) {
    return (unsigned long long)((unsigned)__float_as_int(v) & 0x7FFFFFFFu);
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// IEEE bit patterns of non-negative values order like the values (NaN above +Inf), so an
// integer max over |x| bits is the max-norm and propagates NaN.
__global__ void maxabs_kernel(const RedBatch b, unsigned long long* out) {
    const RedField F = b.f[blockIdx.y];
    // warp tasks of up to 256 consecutive elements of one row: one 32-bit division per task, and
    // a lane keeps up to 8 independent loads in flight
    constexpr int kW = 256;
    const int nch = (F.n0 + kW - 1) / kW;
    const int ntask = nch * F.n1 * F.n2;
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long m = 0;
    for (int task = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; task < ntask; task += nw) {
        const int row = task / nch, c = task - row * nch;
        const int k = row / F.n1, j = row - k * F.n1;
        const long base = (long)j * F.s1 + (long)k * F.s2;
        const int i0 = c * kW + lane, i1 = min(F.n0, (c + 1) * kW);
        if (F.is64) {
            const double* q = static_cast<const double*>(F.p) + base;
#pragma unroll
            for (int u = 0; u < kW / 32; ++u) {
                const int i = i0 + 32 * u;
                if (i < i1) {
                    const unsigned long long v = abs_bits(q[i]);
                    m = v > m ? v : m;
                }
            }
        } else {
            const float* q = static_cast<const float*>(F.p) + base;
#pragma unroll
            for (int u = 0; u < kW / 32; ++u) {
                const int i = i0 + 32 * u;
                if (i < i1) {
                    const unsigned long long v = abs_bits(q[i]);
                    m = v > m ? v : m;
                }
            }
        }
    }
    m = warp_max_u64(m);
    __shared__ unsigned long long sm[32];
    const int w = threadIdx.x >> 5;
    if (lane == 0) sm[w] = m;
    __syncthreads();
    if (w == 0) {
        m = lane < (int)(blockDim.x >> 5) ? sm[lane] : 0ull;
        m = warp_max_u64(m);
        if (lane == 0) atomicMax(out + blockIdx.y, m);
    }
}

}  // namespace

// Enqueue the reduction of `nfields` fields into ctx->d_red[0..nfields).
int cg_maxabs_enqueue(cg_ctx* ctx, int nfields, const cg_field* fields) {
    if (nfields < 1 || nfields > kMaxRedFields)
        return cg_fail(ctx, CG_ERR_ARG, "cg_maxabs: nfields %d not in 1..%d", nfields, kMaxRedFields);
    RedBatch b;
    std::memset(&b, 0, sizeof(b));
    b.nfields = nfields;
    long biggest = 1;
    for (int i = 0; i < nfields; ++i) {
        const cg_field& f = fields[i];
        if (!f.data || (f.dtype != CG_F32 && f.dtype != CG_F64) || f.ndim < 1 || f.ndim > 3)
            return cg_fail(ctx, CG_ERR_ARG, "cg_maxabs: field %d invalid", i);
        const int esz = f.dtype == CG_F64 ? 8 : 4;
        long off = cg_origin_offset(f);
        for (int d = 0; d < f.ndim; ++d) off += f.stride[d];  // logical index 1 along each dim
        RedField& R = b.f[i];
        R.p = static_cast<const char*>(f.data) + off * esz;
        R.s1 = f.ndim > 1 ? f.stride[1] : 0;
        R.s2 = f.ndim > 2 ? f.stride[2] : 0;
        R.n0 = f.n[0];
        R.n1 = f.ndim > 1 ? f.n[1] : 1;
        R.n2 = f.ndim > 2 ? f.n[2] : 1;
        R.is64 = f.dtype == CG_F64;
        biggest = std::max(biggest, (long)R.n0 * R.n1 * R.n2);
    }
    CG_CUDA(ctx, cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long) * nfields, ctx->stream));
    const int threads = 512;
    int blocks = (int)std::min<long>(cg_div_up(biggest, threads), (long)ctx->num_sms * 4);
    blocks = std::max(blocks, 1);
    maxabs_kernel<<<dim3(blocks, nfields), threads, 0, ctx->stream>>>(b, ctx->d_red);
    CG_CHECK_LAUNCH(ctx);
    return CG_OK;
}

// Copy the reduction slots to the host and decode them.
int cg_maxabs_collect(cg_ctx* ctx, int nfields, const cg_field* fields, double* out, int32_t* nonfinite) {
    CG_CUDA(ctx, cudaMemcpyAsync(ctx->h_red, ctx->d_red, sizeof(unsigned long long) * nfields,
                                 cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int bad = 0;
    for (int i = 0; i < nfields; ++i) {
        const unsigned long long v = ctx->h_red[i];
        if (fields[i].dtype == CG_F64) {
            double x;
            std::memcpy(&x, &v, 8);
            out[i] = x;
            if (v >= 0x7FF0000000000000ull) bad = 1;
        } else {
            const unsigned u = (unsigned)v;
            float x;
            std::memcpy(&x, &u, 4);
            out[i] = (double)x;
            if (u >= 0x7F800000u) bad = 1;
        }
    }
    if (nonfinite) *nonfinite = bad;
    return CG_OK;
}

extern "C" int cg_maxabs(cg_ctx* ctx, int nfields, const cg_field* fields, double* out_host, int32_t* nonfinite) {
    if (!ctx) return cg_fail(nullptr, CG_ERR_ARG, "cg_maxabs: ctx is NULL");
    if (!fields || !out_host) return cg_fail(ctx, CG_ERR_ARG, "cg_maxabs: NULL argument");
    cudaSetDevice(ctx->device);
    int rc = cg_maxabs_enqueue(ctx, nfields, fields);
    if (rc) return rc;
    return cg_maxabs_collect(ctx, nfields, fields, out_host, nonfinite);
}

// ---- max-norm without any allocation ----------------------------------------------------------
//
// For callers that cannot allocate device memory: a host runtime that owns all device memory
// through its own pool and forbids a library's cudaMalloc (a Julia or Python runtime with a
// caching allocator, for instance), or an embedded deployment with a fixed device-memory
// budget. The reduction slots live in this file-scope device array instead of a context's
// buffer. Every GPU that loads the library holds these 128 bytes until the process exits.

constexpr int kNoAllocMaxFields = CG_MAXABS_NOALLOC_MAX_FIELDS;
static_assert(kNoAllocMaxFields <= kMaxRedFields, "the allocation-free slots must fit one RedBatch");
static __device__ __align__(256) unsigned long long g_noalloc_red[kNoAllocMaxFields];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned long long* g_noalloc_addr[kNoAllocMaxDevices] = {};  // device address per device

// errors of this context-free entry go to the calling thread's own message buffer
template <typename... A>
int noalloc_fail(int code, const char* fmt, A... args) {
    return cg_fail(nullptr, code, fmt, args...);
}
}  // namespace

extern "C" int cg_maxabs_noalloc(int device, void* stream, int nfields, const cg_field* fields, double* out_host,
                                 int32_t* nonfinite) {
    if (!fields || !out_host) return noalloc_fail(CG_ERR_ARG, "cg_maxabs_noalloc: NULL argument");
    if (nfields < 1 || nfields > kNoAllocMaxFields)
        return noalloc_fail(CG_ERR_ARG, "cg_maxabs_noalloc: nfields %d outside 1..%d (the fixed scratch holds %d slots)",
                            nfields, kNoAllocMaxFields, kNoAllocMaxFields);
    if (device < 0 || device >= kNoAllocMaxDevices)
        return noalloc_fail(CG_ERR_ARG, "cg_maxabs_noalloc: device %d outside 0..%d", device, kNoAllocMaxDevices - 1);
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return noalloc_fail(CG_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
    auto restore = [&]() {
        if (prev >= 0 && prev != device) cudaSetDevice(prev);
    };
    // one-time set-up per device (with that device current): the host-side name of the array
    // is not a device address, so fetch the device address of the symbol
    unsigned long long* slots = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[device]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_red);
            if (e != cudaSuccess) {
                restore();
                return noalloc_fail(CG_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            }
            g_noalloc_addr[device] = static_cast<unsigned long long*>(p);
        }
        slots = g_noalloc_addr[device];
    }
    RedBatch b;
    std::memset(&b, 0, sizeof(b));
    b.nfields = nfields;
    long biggest = 1;
    for (int i = 0; i < nfields; ++i) {
        const cg_field& f = fields[i];
        if (!f.data || (f.dtype != CG_F32 && f.dtype != CG_F64) || f.ndim < 1 || f.ndim > 3) {
            restore();
            return noalloc_fail(CG_ERR_ARG, "cg_maxabs_noalloc: field %d invalid", i);
        }
        const int esz = f.dtype == CG_F64 ? 8 : 4;
        long off = cg_origin_offset(f);
        for (int d = 0; d < f.ndim; ++d) off += f.stride[d];
        RedField& R = b.f[i];
        R.p = static_cast<const char*>(f.data) + off * esz;
        R.s1 = f.ndim > 1 ? f.stride[1] : 0;
        R.s2 = f.ndim > 2 ? f.stride[2] : 0;
        R.n0 = f.n[0];
        R.n1 = f.ndim > 1 ? f.n[1] : 1;
        R.n2 = f.ndim > 2 ? f.n[2] : 1;
        R.is64 = f.dtype == CG_F64;
        biggest = std::max(biggest, (long)R.n0 * R.n1 * R.n2);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the call ends by synchronising the stream to hand the maxima to the host; on a stream
    // that is being captured that would fail and void the caller's capture, so refuse first
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        restore();
        return noalloc_fail(CG_ERR_ARG, "cg_maxabs_noalloc: the stream is being captured (or cannot be queried: %s); "
                            "the call blocks until the maxima are on the host",
                            cudaGetErrorString(e));
    }
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    // the slots keep the previous call's maxima: clear them first
    e = cudaMemsetAsync(slots, 0, sizeof(unsigned long long) * nfields, st);
    if (e == cudaSuccess) {
        const int threads = 512;
        const int blocks = std::max(1, (int)std::min<long>(cg_div_up(biggest, threads), (long)sms * 4));
        maxabs_kernel<<<dim3(blocks, nfields), threads, 0, st>>>(b, slots);
        e = cudaGetLastError();
    }
    unsigned long long host_bits[kNoAllocMaxFields];
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host_bits, slots, sizeof(unsigned long long) * nfields, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    restore();
    if (e != cudaSuccess) return noalloc_fail(CG_ERR_CUDA, "cg_maxabs_noalloc: %s", cudaGetErrorString(e));
    int bad = 0;
    for (int i = 0; i < nfields; ++i) {
        const unsigned long long v = host_bits[i];
        if (fields[i].dtype == CG_F64) {
            double x;
            std::memcpy(&x, &v, 8);
            out_host[i] = x;
            if (v >= 0x7FF0000000000000ull) bad = 1;
        } else {
            const unsigned u = (unsigned)v;
            float x;
            std::memcpy(&x, &u, 4);
            out_host[i] = (double)x;
            if (u >= 0x7F800000u) bad = 1;
        }
    }
    if (nonfinite) *nonfinite = bad;
    return CG_OK;
}
