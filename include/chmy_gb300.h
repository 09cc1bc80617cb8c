/*
 * chmy_gb300.h — C ABI of libchmy_gb300.so, the GB300 (sm_103a) implementation of
 * Chmy.jl's staggered-grid finite-difference hot path.
 *
 * Every entry point is `extern "C"`, takes plain pointers, sizes and POD descriptors,
 * returns an int status (CG_OK = 0) and never throws or aborts. A failing call records a
 * message retrievable with cg_last_error(). Work is stream-ordered on the context's
 * stream (cg_set_stream); cg_sync() gives the blocking semantics of Chmy's Launcher,
 * which synchronizes after every launch (Chmy.jl src/KernelLaunch.jl:117).
 *
 * Memory layout (identical to Chmy.Field, src/Fields/field.jl:6-22,56-62): a field of
 * logical extent n_d per dimension (n cells at Center, n+1 at Vertex, src/Grids/
 * abstract_axis.jl:47-50) and halo H_d is stored with padded extent n_d + 4 H_d, x fastest.
 * Logical index I_d (1-based like Julia, valid range 1-2H_d .. n_d+2H_d) lives at element
 *     data[ sum_d (I_d + 2 H_d - 1) * stride[d] ].
 * A dense Chmy array has stride = (1, nx+4Hx, (nx+4Hx)(ny+4Hy)); pitched layouts (padded
 * rows for aligned vector loads) are expressed through larger strides. All kernels need
 * H_d >= 1 in every used dimension.
 */
#ifndef CHMY_GB300_H
#define CHMY_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define CG_API __attribute__((visibility("default")))
#else
#define CG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define CG_ABI_VERSION 3

/* ---- status codes --------------------------------------------------------------- */
enum {
    CG_OK            = 0,
    CG_ERR_ARG       = 1, /* bad pointer, size, dtype, location or halo                  */
    CG_ERR_CUDA      = 2, /* a CUDA runtime call failed (message holds cudaGetErrorString) */
    CG_ERR_NONFINITE = 3, /* a residual or field contains NaN/Inf                          */
    CG_ERR_TIMEOUT   = 4, /* a bounded device-side wait ran out                            */
    CG_ERR_UNSUPPORTED = 5, /* valid request outside what this build implements           */
    CG_ERR_NOCONV    = 6  /* iterative solve hit its iteration cap before the tolerance   */
};

/* ---- element types and locations ---------------------------------------------------- */
enum { CG_F32 = 1, CG_F64 = 2 };
enum { CG_CENTER = 0, CG_VERTEX = 1 }; /* Chmy.Grids.Center / Vertex (src/Grids/Grids.jl:33,40) */

/* ---- boundary-condition kinds (src/BoundaryConditions/first_order_boundary_condition.jl) */
enum {
    CG_BC_NONE      = 0, /* `nothing` in a Chmy batch: side untouched                       */
    CG_BC_DIRICHLET = 1, /* FirstOrderBC{DirichletKind}, constant value                     */
    CG_BC_NEUMANN   = 2, /* FirstOrderBC{NeumannKind}, constant flux                        */
    CG_BC_PERIODIC  = 3  /* ghost <- opposite interior (both sides of a dimension at once)  */
};

/* A field view. `data` is the start of the padded allocation (see the layout note). */
typedef struct cg_field {
    void*   data;
    int32_t dtype;     /* CG_F32 or CG_F64                                   */
    int32_t ndim;      /* 1, 2 or 3                                          */
    int32_t n[3];      /* logical extent per dim (unused dims: 1)            */
    int32_t loc[3];    /* CG_CENTER / CG_VERTEX per dim                       */
    int32_t halo[3];   /* H per dim (Chmy default 1; unused dims: 0)          */
    int32_t pad_;
    int64_t stride[3]; /* element strides, stride[0] == 1; unused dims: 0     */
} cg_field;

/* A UniformGrid (src/Grids/structured_grid.jl:27-39, src/Grids/uniform_axis.jl:1-31).
 * spacing = extent / n and inv_spacing = 1 / spacing are computed by the caller in the
 * grid's element type (Float32 grids round both to float) and passed here exactly. */
typedef struct cg_grid {
    int32_t ndim;
    int32_t n[3];          /* cells per dim (unused dims: 1) */
    double  origin[3];
    double  extent[3];
    double  spacing[3];
    double  inv_spacing[3];
} cg_grid;

/* Boundary conditions of one field: kind and value per dimension and side (side 0 =
 * Side(1) = left, side 1 = Side(2) = right). Dirichlet value `nothing` and Neumann value
 * `nothing` are 0 (first_order_boundary_condition.jl:34).
 * values[d][s]: NULL, or per-point values that replace value[d][s]. These are Chmy's
 * Field-valued conditions, value(bc::FirstOrderBC{<:AbstractField}, ...) =
 * bc.value[remove_dim(dim, I)...] (first_order_boundary_condition.jl:38-40), and
 * BoundaryFunction values evaluated at the condition's points (boundary_function.jl:34-44).
 * The array has the field's element type over the logical indices 0..n_t+2 of the grid's
 * other dimensions, in ascending dimension order with the first fastest, so
 * (n_t0 + 3) x (n_t1 + 3) values in 3D and n_t0 + 3 in 2D. It is device memory for the library
 * and host memory for the oracle. */
typedef struct cg_bc {
    int32_t kind[3][2];
    double  value[3][2];
    const void* values[3][2];
} cg_bc;

/* FieldMask (src/GridOperators/field_mask.jl:1-117): one weight field per location. at[m] is
 * the mask at the location whose bit d is set for Vertex along dimension d (2D: 0 = (C,C),
 * 1 = (V,C), 2 = (C,V), 3 = (V,V); 3D up to 7 = (V,V,V)). Entries an operation does not read
 * may be empty. A masked operator multiplies every operand value by the mask at the operand's
 * location and index (src/GridOperators/masked_operators.jl:11-39). */
typedef struct cg_mask {
    cg_field at[8];
} cg_mask;

typedef struct cg_ctx cg_ctx;

/* ---- context and memory ----------------------------------------------------------- */

/* Library ABI version (CG_ABI_VERSION). */
CG_API int cg_abi_version(void);

/* Arch(backend; device_id) + activate! (src/Architectures.jl:46-49,71-74): binds the calling
 * thread to `device` (0-based CUDA ordinal; Chmy's device_id is 1-based) and creates a
 * context with its own stream. The stream is a blocking one, ordered with work on the legacy
 * default stream (host-side copies of PyTorch's default stream, for instance); cg_set_stream
 * replaces it. */
CG_API int cg_init(int device, cg_ctx** out);
CG_API int cg_destroy(cg_ctx* ctx);
/* Message of the last failing call on `ctx`. With ctx == NULL: the calling thread's last
 * failure of a call that takes no context (cg_init, cg_maxabs_noalloc, ...). */
CG_API const char* cg_last_error(const cg_ctx* ctx);
/* Use `stream` (a cudaStream_t; NULL restores the context's own stream) for later calls. */
CG_API int cg_set_stream(cg_ctx* ctx, void* stream);
/* KernelAbstractions.synchronize(backend) (src/KernelLaunch.jl:117). */
CG_API int cg_sync(cg_ctx* ctx);

/* Field(backend, grid, loc, T; halo) storage (src/Fields/field.jl:56-62): zero-filled,
 * dense Chmy layout when `pitch_align` is 0, otherwise rows padded so that logical x index
 * 0 of every row starts on a `pitch_align`-byte boundary (a power of two >= 16). */
CG_API int cg_field_alloc(cg_ctx* ctx, int dtype, int ndim, const int32_t n[3], const int32_t loc[3],
                   const int32_t halo[3], int pitch_align, cg_field* out);
CG_API int cg_field_free(cg_ctx* ctx, cg_field* f);
/* Copies between a dense host array holding the whole padded field and the device field. */
CG_API int cg_field_upload(cg_ctx* ctx, const cg_field* f, const void* host_dense);
CG_API int cg_field_download(cg_ctx* ctx, const cg_field* f, void* host_dense);

/* The device's FP64 FMA throughput (FLOP/s, 2 per FMA), measured with CUDA events on the
 * context's stream: the roofline denominator of the kernels bound by the FP64 pipe. A measuring
 * aid with no counterpart in the reference. */
CG_API int cg_fp64_peak(cg_ctx* ctx, double* flops);

/* ---- boundary conditions ---------------------------------------------------------- */

/* bc!(arch, grid, batch) for a FieldBatch of `nfields` fields
 * (src/BoundaryConditions/batch.jl:104-113,247-268). The result equals Chmy's 2N
 * per-side launches applied Dim N -> 1, Side 1 then 2, over tangential indices
 * 0 .. n+2, but runs as ONE launch: each boundary point's final value is evaluated
 * through its chain of ghost rules. */
CG_API int cg_bc_apply(cg_ctx* ctx, const cg_grid* grid, int nfields, const cg_field* fields,
                const cg_bc* bcs);

/* ---- reductions --------------------------------------------------------------------- */

/* maximum(abs.(interior(f))) for each of `nfields` fields, as used by the PT convergence
 * checks (e.g. examples/stokes_2d_inc_ve_T.jl:155-157). One launch; `out_host[i]` gets the
 * maximum (NaN if any interior value is NaN); `*nonfinite` is set to 1 if any value is
 * NaN or Inf. Blocks until the values are on the host. */
CG_API int cg_maxabs(cg_ctx* ctx, int nfields, const cg_field* fields, double* out_host,
              int32_t* nonfinite);

/* The same max-norm reduction for callers that cannot allocate device memory: a host
 * runtime that owns all device memory through its own pool and does not let a library call
 * cudaMalloc (a Julia or Python runtime with a caching allocator, for instance), or a
 * deployment with a fixed device-memory budget. It needs no context and calls no
 * cudaMalloc/cudaFree (nor any allocating library routine): its reduction slots are a fixed
 * array of CG_MAXABS_NOALLOC_MAX_FIELDS 64-bit words in the library's device memory, which
 * every GPU that loads the library keeps until exit.
 * This entry point has no counterpart in the reference.
 * - `device`: CUDA ordinal to run on (made current for the call, then restored); `stream`:
 *   a cudaStream_t or NULL. The call blocks until the values are on the host (it
 *   synchronises `stream`); a stream that is being captured is rejected with CG_ERR_ARG
 *   before anything is enqueued.
 * - nfields above CG_MAXABS_NOALLOC_MAX_FIELDS is rejected with CG_ERR_ARG.
 * - The first call on a device looks up the array's device address (once per device, with
 *   that device current); make that first call before any stream capture.
 * - All calls share the array (the slots are cleared at the start of each call): calls
 *   that overlap on the GPU race and must not be issued concurrently.
 * Errors are reported through cg_last_error(NULL), per calling thread. */
#define CG_MAXABS_NOALLOC_MAX_FIELDS 16
CG_API int cg_maxabs_noalloc(int device, void* stream, int nfields, const cg_field* fields,
                             double* out_host, int32_t* nonfinite);

/* ---- explicit diffusion (examples/diffusion_2d.jl:8-19, diffusion_2d_perf.jl:11-23) -- */

/* compute_q!: q.d = -chi * d(C)/dx_d at I in [0, n+1]^N. `q` holds ndim face fields. */
CG_API int cg_diffusion_compute_q(cg_ctx* ctx, const cg_grid* grid, const cg_field* q,
                           const cg_field* C, double chi);
/* update_C!: C -= dt * divg(q) at I in [0, n+1]^N. */
CG_API int cg_diffusion_update_C(cg_ctx* ctx, const cg_grid* grid, const cg_field* C,
                          const cg_field* q, double dt);
/* One fused step: C_out = C_in - dt*divg(-chi*grad C_in) over [0, n+1]^N, followed by
 * bc!(C_out => bc). Equals compute_q! + update_C! + bc! with freshly zeroed q arrays.
 * C_out and C_in must not alias (ping-pong buffers); their outer halos must match. */
CG_API int cg_diffusion_step(cg_ctx* ctx, const cg_grid* grid, const cg_field* C_out,
                      const cg_field* C_in, double chi, double dt, const cg_bc* bc);
/* `nsteps` fused steps ping-ponging between A and B (result in A if nsteps is even,
 * else in B), captured once into a CUDA graph and replayed. */
CG_API int cg_diffusion_run(cg_ctx* ctx, const cg_grid* grid, const cg_field* A, const cg_field* B,
                     double chi, double dt, const cg_bc* bc, int nsteps);

/* The same with the masked operators: q.d = -chi * ∂d(C, ω) and C -= dt * divg(q, ω)
 * (masked_field_operators.jl:20-57): the Center mask at[0] weighs C, the d-face mask at[1 << d]
 * weighs q.d. No reference example runs them; the oracle restates the operators. */
CG_API int cg_diffusion_compute_q_masked(cg_ctx* ctx, const cg_grid* grid, const cg_field* q,
                                         const cg_field* C, double chi, const cg_mask* mask);
CG_API int cg_diffusion_update_C_masked(cg_ctx* ctx, const cg_grid* grid, const cg_field* C,
                                        const cg_field* q, double dt, const cg_mask* mask);
/* nsteps fused masked steps A -> B -> A ... with bc!(C => bc) after each, one CUDA graph. */
CG_API int cg_diffusion_run_masked(cg_ctx* ctx, const cg_grid* grid, const cg_field* A, const cg_field* B,
                                   double chi, double dt, const cg_bc* bc, const cg_mask* mask, int nsteps);

/* ---- adjoint of the explicit diffusion loop (no reference counterpart: the reference has no
 * adjoint) --------------------------------------------------------------------------------
 * The loop C^{n+1} = bc!(C^n - dt divg(-chi grad C^n)) of cg_diffusion_run, differentiated for a
 * misfit J(C^N) of the final interior: dJ/dC^0 at the interior cells and dJ/dchi. The ghost
 * cells follow the interior through the boundary rules, so every side must carry a Dirichlet,
 * Neumann or Periodic rule (CG_ERR_UNSUPPORTED otherwise); the fields are at Center. */

/* Bytes of a tape of `nsteps` steps for a C of this layout: a 256-byte header, then the states
 * C^0 .. C^nsteps, each C's padded allocation rounded up to 256 bytes. No context, no device work. */
CG_API int cg_diffusion_tape_bytes(const cg_grid* grid, const cg_field* C, int nsteps, size_t* bytes);
/* cg_diffusion_run's loop (the same steps, bit for bit) that records every state on `tape`
 * (device memory of at least cg_diffusion_tape_bytes, 256-byte aligned): on entry C holds C^0
 * with its ghost cells set by bc!, on return C^nsteps. */
CG_API int cg_diffusion_run_taped(cg_ctx* ctx, const cg_grid* grid, const cg_field* C, double chi, double dt,
                                  const cg_bc* bc, int nsteps, void* tape, size_t tape_bytes);
/* The reverse sweep over a tape of cg_diffusion_run_taped: on entry lam holds dJ/dC^N at the
 * interior cells, on return dJ/dC^0 there (the ghost cells' dependence folded in); dJ (host, may
 * be NULL) gains dJ/dchi in dJ[0]. lam and work have C's layout (work is overwritten); chi, dt
 * and the boundary kinds must be the taped run's (the tape's header is checked). Per step the
 * reverse kernel applies the transposed stencil in gather form and adds lam (C^{n+1} - C^n) to a
 * per-cell FP64 sum; the sums are added once, in a fixed order, at the end (dJ/dchi is
 * reproducible bit for bit). The call synchronises the stream. */
CG_API int cg_diffusion_adjoint_run(cg_ctx* ctx, const cg_grid* grid, const void* tape, size_t tape_bytes,
                                    const cg_field* lam, const cg_field* work, double chi, double dt, const cg_bc* bc,
                                    double* dJ);

/* ---- viscoelastic Stokes (examples/stokes_{2,3}d_inc_ve_T.jl) ---------------------- */

/* Field set of the VE Stokes examples. Tensor order: 2D (xx, yy, xy); 3D (xx, yy, zz,
 * xy, xz, yz) at the TensorField locations of src/Fields/field.jl:182-206.
 * Optional fields have data == NULL:
 *   eta      Center viscosity. NULL: scalar params.eta / params.eta_ve, arithmetic exactly
 *            as in the examples. Present (variable-viscosity extension; the examples have a
 *            scalar eta), with ieta = 1/eta, inv_Gdt = 1/(G dt), eta_ve = 1/(ieta + inv_Gdt):
 *              diagonal tau and P use the cell's ieta;
 *              shear tau uses ieta linearly interpolated (Chmy `lerp` rule) to its edge,
 *              i.e. the harmonic (`hlerp`-type) average of the surrounding viscosities;
 *              r_tau = -(tau - tau_old)*inv_Gdt - tau*ieta + 2(eps - divV/3);
 *              the velocity PT step is V += r_V * (nu_dtau * (min(ieta_l, ieta_r) + inv_Gdt)),
 *              i.e. nu_dtau / max(eta_ve) of the two cells beside the face.
 *   inv_eta  Center 1/eta precomputed by the caller (optional; bit-identical to computing
 *            1/eta in the kernel, saves the divisions).
 *   rho_g[d] body force subtracted from r_V.d (the examples use only the last component).
 *   r_V, divV are written every call unless NULL.                                       */
typedef struct cg_stokes_fields {
    cg_field V[3];
    cg_field r_V[3];
    cg_field P;
    cg_field divV;
    cg_field tau[6];
    cg_field tau_old[6];
    cg_field eta;
    cg_field inv_eta;
    cg_field rho_g[3];
    cg_field T;
    cg_field T_old;
    cg_field qT[3];
} cg_stokes_fields;

/* Scalars of the PT loop (examples/stokes_2d_inc_ve_T.jl:86-93,142). */
/* A FunctionField evaluated on the device (src/Fields/function_field.jl:49-59, the Continuous
 * form): the value at logical index I is func(coord(grid, loc, I)..., parameters...), computed
 * by the kernel that uses it instead of loaded from an array. Coordinates follow
 * src/Grids/uniform_axis.jl: Vertex muladd(I-1, Δ, o), Center muladd(I-1, Δ, muladd(0.5, Δ, o)),
 * in the kernel's precision. The functions a kernel can evaluate (p = parameters):
 *   CG_FN_NONE    no function
 *   CG_FN_CONST   p[0]
 *   CG_FN_BALL    ifelse(sum_d (x_d - p[d])^2 < p[3]^2, p[4], p[5]), the squares summed in
 *                 dimension order: init_incl of examples/stokes_2d_inc_ve_T.jl:106 (x0 = p[0],
 *                 y0 = p[1], z0 = p[2], r = p[3], in = p[4], out = p[5])
 *   CG_FN_AFFINE  p[0] + p[1] x + p[2] y + p[3] z, left to right */
enum { CG_FN_NONE = 0, CG_FN_CONST = 1, CG_FN_BALL = 2, CG_FN_AFFINE = 3 };
typedef struct cg_function {
    int32_t kind;
    int32_t pad_;
    double  p[8];
} cg_function;

typedef struct cg_stokes_params {
    double eta;          /* scalar viscosity (used when fields.eta.data == NULL)       */
    double eta_ve;       /* 1/(1/eta + 1/(G dt)) (scalar case)                          */
    double G;
    double dt;
    double dtau_Pr;
    double dtau_r;
    double nu_dtau;
    double lambda_rhoCp; /* thermal diffusivity for the thermal kernels                  */
    /* Body force of component d as a device FunctionField at V.d's location (Vertex along d),
     * e.g. rho_g_fn[1] = the examples' rhogy = FunctionField(init_incl, grid, (Center(),
     * Vertex()); ...) (examples/stokes_2d_inc_ve_T.jl:107). The velocity update and the
     * residuals subtract it like an array rho_g[d]; a component takes an array or a function,
     * not both. The fused ping-pong entry (cg_stokes_pt_iterations_pp) reads arrays only. */
    cg_function rho_g_fn[3];
} cg_stokes_params;

/* set!(f, grid, func) for a device FunctionField: f (any location) gets func at every padded
 * point (logical 1-2H .. n+2H), evaluated on the device. */
CG_API int cg_function_fill(cg_ctx* ctx, const cg_grid* grid, const cg_function* fn, const cg_field* f);

/* BoundaryFunction values evaluated on the device (src/BoundaryConditions/boundary_function.jl:
 * 11-44, the continuous form), per field, dimension and side. A side whose fn kind is not
 * CG_FN_NONE takes its value at each point the condition writes from the function instead of
 * cg_bc.value / cg_bc.values: func(x...) at coord(grid, L, I...) with I the written point (the
 * boundary node for Dirichlet on a Vertex dimension, else the ghost) and L the field's location
 * along the dimension for Dirichlet and its flip for Neumann, used for every dimension
 * (first_order_boundary_condition.jl:46-84); with full_dims 0 (Chmy's reduce_dims=true) the
 * coordinate along the condition's dimension is left out of x. Coordinates and the function are
 * evaluated in the field's precision with fused multiply-adds, as for cg_function. */
typedef struct cg_bc_fn {
    cg_function fn[3][2];
    int32_t full_dims[3][2];
} cg_bc_fn;
/* cg_bc_apply with BoundaryFunction sides: fns[i] belongs to fields[i] (fns may be NULL). */
CG_API int cg_bc_apply_fn(cg_ctx* ctx, const cg_grid* grid, int nfields, const cg_field* fields,
                          const cg_bc* bcs, const cg_bc_fn* fns);

/* update_old!: T_old = T; tau_old = tau at I in [0, n+1]^N. */
CG_API int cg_stokes_update_old(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f);
/* update_stress!: strain rates, divV, P and tau PT update at I in [0, n+1]^N. */
CG_API int cg_stokes_update_stress(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                            const cg_stokes_params* p);
/* update_velocity!: r_V and V PT update at I in [0, n+1]^N (no bc; see cg_bc_apply). */
CG_API int cg_stokes_update_velocity(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                              const cg_stokes_params* p);
/* update_thermal_flux! and update_thermal! (examples/stokes_2d_inc_ve_T.jl:45-60). */
CG_API int cg_stokes_update_thermal_flux(cg_ctx* ctx, const cg_grid* grid,
                                  const cg_stokes_fields* f, const cg_stokes_params* p);
CG_API int cg_stokes_update_thermal(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                             const cg_stokes_params* p);

/* `niter` PT iterations: update_stress!, update_velocity!, bc!(V => bc_V[d]) each, captured
 * into a CUDA graph per (fields, niter) and replayed. divV and r_V are written only on the
 * last iteration (they are only read by the convergence check). */
CG_API int cg_stokes_pt_iterations(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                            const cg_stokes_params* p, const cg_bc* bc_V, int niter);

/* The same kernels with Chmy's masked operators (src/GridOperators/masked_operators.jl:11-39,
 * masked_field_operators.jl), as a user writes them with a FieldMask ω (docs/src/concepts/
 * grid_operators.md "Masking"): update_stress! with ∂(V.d, ω, g, I) for every strain rate and
 * divg(V, ω, g, I); update_velocity! with ∂(Pr, ω, g, I) and ∂(τ.c, ω, g, I). Each operand of a
 * derivative is multiplied by the mask at its own location and index; the viscosity terms, the
 * stress's own values and the body force are not masked. Mask entries read (cg_mask.at by
 * location bits): update_stress! the velocity locations 1 << d; update_velocity! the cell (0)
 * and the shear locations (2D: 3; 3D: 3, 5, 6); the PT chunk both. With unit weights the
 * results equal the unmasked entries' bit for bit. */
CG_API int cg_stokes_update_stress_masked(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                          const cg_stokes_params* p, const cg_mask* mask);
CG_API int cg_stokes_update_velocity_masked(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                            const cg_stokes_params* p, const cg_mask* mask);
CG_API int cg_stokes_pt_iterations_masked(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                          const cg_stokes_params* p, const cg_bc* bc_V, const cg_mask* mask,
                                          int niter);

/* Ping-pong form of cg_stokes_pt_iterations for 2D and 3D variable viscosity. Each
 * iteration is one fused launch: update_stress! and update_velocity! together, in a kernel
 * that marches over rows (2D) or planes (3D). It reads V, P, tau from `a` and writes them to
 * `b`, then from `b` to `a`, and each launch is followed by bc!(V). `niter` must be even (the
 * result is in `a`; `b` holds the state one iteration earlier). Points outside the launch range
 * [0, n+1]^N are never written: `a` and `b` must agree there (b a copy of a, for instance), as
 * the in-place reference loop keeps one value per point. In 2D the autotuner may take two
 * iterations per launch (a kernel that keeps the intermediate state in registers) where no
 * bc!(V) launch is needed between iterations; the results are the same bits. All other fields (tau_old, inv_eta, rho_g, divV, r_V) are taken from
 * `a`; inv_eta is required. divV and r_V are written on the last iteration. Every operation
 * is rounded once, in the order of the reference kernels, with no contraction into FMA: the
 * values are those of a CPU evaluation with -ffp-contract=off. */
CG_API int cg_stokes_pt_iterations_pp(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* a,
                                      const cg_stokes_fields* b, const cg_stokes_params* p,
                                      const cg_bc* bc_V, int niter);

/* Convergence measures of examples/stokes_2d_inc_ve_T.jl:154-157: applies
 * bc!(r_V.d => Dirichlet on dim d) and returns err[0] = max|divV| * tau_scale,
 * err[1 + d] = max|r_V.d| * v_scale. Blocks. */
CG_API int cg_stokes_residual(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                       double tau_scale, double v_scale, double* err_host);

/* PT solve options and result. */
typedef struct cg_solve_opts {
    int32_t max_iter;    /* niter                                                        */
    int32_t ncheck;      /* iterations between convergence checks                         */
    double  eps;         /* tolerance on every err component                              */
    double  tau_scale;   /* err[0] = max|divV| * tau_scale                                */
    double  v_scale;     /* err[1..] = max|r_V| * v_scale                                 */
    int32_t precision;   /* CG_F64: plain FP64 PT; CG_F32: FP32 PT inside FP64 defect
                            correction (fields stay FP64; FP32 work arrays are internal)  */
    int32_t max_outer;   /* defect-correction cycles (precision == CG_F32)                */
    double  inner_rtol;  /* FP32 inner solve stops at this residual reduction              */
} cg_solve_opts;

typedef struct cg_solve_result {
    int32_t iterations;       /* total PT iterations (FP32 + FP64)                         */
    int32_t outer;            /* defect-correction cycles used                             */
    int32_t checks;
    int32_t converged;
    double  err[4];           /* last FP64 convergence measures                            */
    double  seconds;          /* device time of the solve (CUDA events)                    */
    double  err_tau;          /* max constitutive residual * tau_scale (precision CG_F32;
                                 part of its convergence test, 0 for CG_F64)               */
} cg_solve_result;

/* Full PT solve of one physical step (examples/stokes_2d_inc_ve_T.jl:144-163) on FP64
 * fields. Returns CG_ERR_NONFINITE on NaN/Inf, CG_ERR_NOCONV when max_iter is reached. */
CG_API int cg_stokes_solve(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                    const cg_stokes_params* p, const cg_bc* bc_V, const cg_solve_opts* o,
                    cg_solve_result* res);

/* ---- adjoint: gradient of a velocity misfit with respect to log-viscosity ------------------
 * For a misfit J(V) of the converged VE Stokes step, the adjoint velocity mu solves the same
 * Stokes problem (the discrete operator is symmetric): cg_stokes_solve on a field set with
 * rho_g = -dJ/dV, tau_old = 0, V = P = tau = 0 initially and the forward's boundary-condition
 * kinds with zero values. This entry then writes, at every interior cell c,
 *   grad_c = dJ/d log(eta_c) = -(1/eta)_c [ eta_ve_c sum_d eps_dd(mu) tau_dd(V)
 *                                           + 1/2 sum_{shear edges e at c} eta_ve_e eps_e(mu) tau_e(V) ]
 * with tau(V) = eta_ve (2 dev(eps(V)) + tau_old/(G dt)) the constitutive stress of the forward's
 * converged velocity `fwd->V` (and `fwd->tau_old` when present), its viscosity `fwd->inv_eta`
 * (else `fwd->eta`), eta_ve = 1/(1/eta + 1/(G dt)) at cells and the edges' 1/eta the
 * Linear-rule mean of their 4 cells, as in the forward kernels. `mu` holds ndim velocity
 * fields. No reference counterpart: the reference has no adjoint. */
CG_API int cg_stokes_gradient_log_eta(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* fwd,
                               const cg_field* mu, const cg_stokes_params* p, const cg_field* grad);

/* ---- thermal coupling (examples/stokes_2d_inc_ve_T.jl:35-60,147-152) ----------------------
 * From the second time step on, every PT iteration of the reference also takes the thermal
 * step: qT_d = -lambda_rhoCp * d_d(T) + max(V_d, 0) * T_left + min(V_d, 0) * T_right
 * (update_thermal_flux!), T = T_old - dt * divg(qT) (update_thermal!), bc!(T => bc_T). */

/* The two thermal kernels fused: T_out = T_old - dt * divg(qT(T, V)) over [0, n+1]^N, with the
 * fluxes computed on the fly and not stored, then bc!(T_out => bc_T) when bc_T is not NULL.
 * f supplies T (read only), T_old and V; p supplies lambda_rhoCp and dt. T_out must not be T.
 * A flux at face index n+2 (beyond the flux kernel's launch range) counts as zero, as a freshly
 * allocated qT reads there. Every operation is rounded once in the reference's order: the
 * values equal a CPU evaluation of the two kernels with -ffp-contract=off. */
CG_API int cg_stokes_thermal_step(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                           const cg_stokes_params* p, const cg_bc* bc_T, const cg_field* T_out);

/* Vector-Jacobian product of the fused thermal step (cg_stokes_thermal_step with bc_T), the
 * transposed stencil of update_thermal_flux! + update_thermal! (no reference counterpart: the
 * reference has no adjoint). For a misfit J of T_out at the interior cells, with mu = dJ/dT_out
 * there, it writes
 *   gT      dJ/dT at the interior cells; T's ghost cells are the bc_T rules' functions of the
 *           interior (T came from a step that ended with bc!(T)), and their terms are folded in
 *           (every side of bc_T must carry a Dirichlet, Neumann or Periodic rule);
 *   gT_old  dJ/dT_old = mu at the interior cells (may be NULL);
 *   gV[d]   dJ/dV.d at the faces an interior cell reads (normal index 1..n+1, tangential 1..n),
 *           with the upwind branches the forward took (max(V, 0) and min(V, 0) both follow V at
 *           V = 0, as the kernel's comparisons do);
 * and dJ (host, may be NULL) gains dJ/dlambda_rhoCp in dJ[0] (summed in FP64 per block of cells
 * and then over the blocks, both in a fixed order; the call then synchronises the stream). f supplies T and V at the step's input;
 * p supplies lambda_rhoCp and dt. */
CG_API int cg_stokes_thermal_step_adjoint(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                          const cg_stokes_params* p, const cg_bc* bc_T, const cg_field* mu,
                                          const cg_field* gT, const cg_field* gT_old, const cg_field* gV, double* dJ);

/* `niter` PT iterations with thermal coupling: update_stress!, update_velocity!, bc!(V), the
 * thermal step and bc!(T), as one graph. T alternates with a library-owned partner buffer and
 * the result is in f->T. */
CG_API int cg_stokes_pt_iterations_thermal(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                                    const cg_stokes_params* p, const cg_bc* bc_V, const cg_bc* bc_T,
                                    int niter);

/* cg_stokes_solve with the thermal step in every PT iteration (the reference's solve for time
 * steps after the first). FP64 PT only: o->precision must be CG_F64. */
CG_API int cg_stokes_solve_thermal(cg_ctx* ctx, const cg_grid* grid, const cg_stokes_fields* f,
                            const cg_stokes_params* p, const cg_bc* bc_V, const cg_bc* bc_T,
                            const cg_solve_opts* o, cg_solve_result* res);

/* ---- pseudo-transient variable-coefficient diffusion -------------------------------------
 * Implicit (backward Euler) diffusion step (C - C_old)/dt = divg(D grad C) solved by damped
 * PT iterations in the pattern of the Stokes PT loop; the flux is Chmy's ∂k∂/divg_grad form
 * q = -lerp(D) ∂C (src/GridOperators/partial_derivatives.jl:14-21). Over I in [0, n+1]^N:
 *   update_q:  q_d += (-(lerp(D -> face_d) * ∂_d C) - q_d) * omega_q
 *   update_C:  R = -(C - C_old) / dt - divg(q);  C += R * dtau_C   (R written if given)
 * then bc!(C => bc). Typical parameters (accelerated PT for diffusion): vdtau = min(Δ)/
 * sqrt(N 1.1), Re = pi + sqrt(pi^2 + l^2/(D_max dt)), theta = l/(Re vdtau),
 * beta = Re D_max/(vdtau l), omega_q = 1/(1 + theta), dtau_C = 1/(beta + 1/dt). */
typedef struct cg_ptdiff_fields {
    cg_field C, C_old, D, q[3];
    cg_field R; /* optional residual output */
} cg_ptdiff_fields;

typedef struct cg_ptdiff_params {
    double dt;
    double omega_q;
    double dtau_C;
} cg_ptdiff_params;

CG_API int cg_ptdiff_update_q(cg_ctx* ctx, const cg_grid* grid, const cg_ptdiff_fields* f,
                              const cg_ptdiff_params* p);
CG_API int cg_ptdiff_update_C(cg_ctx* ctx, const cg_grid* grid, const cg_ptdiff_fields* f,
                              const cg_ptdiff_params* p);
/* `nsteps` implicit steps of `npt` PT iterations each (C_old <- C at the start of every step;
 * bc!(C => bc) after every iteration), replayed from one CUDA graph. R (if given) holds the
 * residual of the last iteration. */
CG_API int cg_ptdiff_run(cg_ctx* ctx, const cg_grid* grid, const cg_ptdiff_fields* f,
                         const cg_ptdiff_params* p, const cg_bc* bc, int nsteps, int npt);

/* One implicit step (C - C_old)/dt = divg(lerp(D) grad C) solved to a tolerance on FP64 fields
 * (3D): C holds the initial guess, C_old the previous step. The measure is
 * err[0] = max |R| dt over the interior cells (logical 1..n), where
 * R = -(C - C_old)/dt - divg(q(C)) and q(C) = -lerp(D) grad C is the exact flux; bc! sets the
 * ghost planes, and every side must carry a Dirichlet or Neumann rule.
 *   o->precision == CG_F64: the PT iterations of cg_ptdiff_run, checked every ncheck.
 *   o->precision == CG_F32: FP64 defect correction. The correction d solves
 *     d/dt - divg(lerp(D) grad d) = R with the rules' homogeneous form, by FP32 PT iterations
 *     (the fused single-pass kernel) on internal FP32 arrays, until its own measure falls
 *     below max(eps/2, inner_rtol err) or stops improving. Then C += d and bc!(C), for at most
 *     max_outer cycles. q is then set to the exact flux of the converged C.
 * Uses max_iter, ncheck, eps, precision, max_outer and inner_rtol of `o`. `res` receives the
 * iteration, check and cycle counts, err[0] and the device time. Returns CG_ERR_NOCONV when
 * the budget runs out and CG_ERR_NONFINITE on NaN/Inf. No reference counterpart: the
 * reference has no solver for this configuration. */
CG_API int cg_ptdiff_solve(cg_ctx* ctx, const cg_grid* grid, const cg_ptdiff_fields* f,
                    const cg_ptdiff_params* p, const cg_bc* bc, const cg_solve_opts* o,
                    cg_solve_result* res);

/* Adjoint of the implicit diffusion steps (no reference counterpart). I - dt L_D is symmetric
 * on the interior cells, so the adjoint of a step is the same step: lambda^n = S lambda^{n+1}
 * is cg_ptdiff_run (1 step) on a field set with C = lambda^{n+1} and zero boundary values. For
 * a misfit J(C^N), dJ/dD = sum over steps of this entry's term, which adds at every interior
 * cell c
 *   scale * sum_{faces f of c} 1/2 (C_r - C_l) idx^2 (lambda_l [l interior] - lambda_r [r interior])
 * (f between cells l and r; a face's D is the mean of its two cells) with lambda = lambda^n,
 * C = C^{n+1} and scale = dt. The reverse sweep needs the states C^{n+1} in reverse order:
 * store them or recompute them from checkpoints (chmy_gb300.adjoint does both). */
CG_API int cg_ptdiff_gradient_D(cg_ctx* ctx, const cg_grid* grid, const cg_field* lam, const cg_field* C,
                                double scale, const cg_field* grad);

/* ---- shallow ice (examples/sia.jl) ----------------------------------------------------- */

/* Parameters of the SIA step. examples/sia.jl:24-54 is Gamma = 1, As = 0.5, n = 3, beta = 0.5,
 * ela = 0.3, m_max = 0.25, dt_max = 0.5 (Δt_mb), cfl = 4.1. The flux of the benchmark
 * ensemble, -Gamma H^(n+2) |∇S|^(n-1) ∇S, is As = 0. */
typedef struct cg_sia_params {
    double  Gamma;  /* coefficient of H^(n+2) in D                                           */
    double  As;     /* coefficient of H^n in D                                               */
    int32_t n;      /* Glen exponent (integer powers by repeated multiplication)             */
    int32_t pad_;
    double  beta;   /* mass balance M = min(beta (S - ela), m_max), S = B + H                */
    double  ela;
    double  m_max;
    double  dt_max; /* Δt = min(min(Δ)^2 / max(interior D) / cfl, dt_max)                    */
    double  cfl;
} cg_sia_params;

/* update_q! (examples/sia.jl:12-16) over the interior cells [1, n]^2 with D evaluated on the
 * fly as the FunctionField of :46-49, D = (Gamma H^(n+2) + As H^n) vmag(∇S)^(n-1),
 * followed by bc!(q.x => (x = Dirichlet()), q.y => (y = Dirichlet())) (:73). B holds the bed
 * over the whole padded array. If dmax_host is not NULL it receives maximum(interior(D)). */
CG_API int cg_sia_update_q(cg_ctx* ctx, const cg_grid* grid, const cg_field* q, const cg_field* H,
                           const cg_field* B, const cg_sia_params* p, double* dmax_host);
/* update_H! (examples/sia.jl:7-10) over [1, n]^2: H = max(H + dt (-divg(q) + M), 0), followed
 * by bc!(H => Neumann()) (:81). */
CG_API int cg_sia_update_H(cg_ctx* ctx, const cg_grid* grid, const cg_field* H, const cg_field* q,
                           const cg_field* B, double dt, const cg_sia_params* p);
/* `nsteps` SIA time steps with the adaptive Δt computed on the device every step (no host
 * synchronisation), replayed from one CUDA graph. q is the flux work array (its final
 * values are those of the last step). `t_host` (optional) receives the simulated time. */
CG_API int cg_sia_run(cg_ctx* ctx, const cg_grid* grid, const cg_field* H, const cg_field* B,
                      const cg_field* q, const cg_sia_params* p, int nsteps, double* t_host);

/* One member of an SIA ensemble: its grid (2D), ice thickness H, bed B and flux work array q. */
typedef struct cg_sia_member {
    cg_grid  grid;
    cg_field H;
    cg_field B;
    cg_field q[2];
} cg_sia_member;

/* `nsteps` SIA time steps of `nmembers` independent solves of uneven grid sizes, each with its
 * own parameters and adaptive Δt (the reference loop of examples/sia.jl:71-81 per member).
 * Every phase of a step is one launch over the tiles of all members; the q and H boundary
 * conditions are folded into the kernels (q.x => (x = Dirichlet()), q.y => (y = Dirichlet()),
 * H => Neumann(), with the reference's corner values; the outer halo is left untouched);
 * the loop is replayed from one CUDA graph. `t_host` (optional, nmembers entries) receives
 * each member's simulated time. All members share one dtype. */
CG_API int cg_sia_ensemble_run(cg_ctx* ctx, int nmembers, const cg_sia_member* members,
                               const cg_sia_params* params, int nsteps, double* t_host);

/* Bytes of an ensemble tape of `nsteps` steps for these members: a 256-byte header, then per
 * step every member's tape in the layout of cg_sia_run_taped. No context, no device work. */
CG_API int cg_sia_ensemble_tape_bytes(int nmembers, const cg_sia_member* members, int nsteps,
                                      size_t* bytes);

/* cg_sia_ensemble_run (same results bit for bit; always the per-phase graph form) that also
 * records every member's reverse-step quantities for each of its `nsteps` (>= 1) steps into
 * `tape` (device memory of at least cg_sia_ensemble_tape_bytes, 256-byte aligned). No
 * reference counterpart. */
CG_API int cg_sia_ensemble_run_taped(cg_ctx* ctx, int nmembers, const cg_sia_member* members,
                                     const cg_sia_params* params, int nsteps, void* tape,
                                     size_t tape_bytes, double* t_host);

/* The reverse sweep over an ensemble tape, all members in each launch: on entry lam[m] holds
 * dJ/dH of member m at its interior cells after the taped run; on return, at its start.
 * dJ (host, 2 per member, may be NULL) gains dJ/dGamma in dJ[2m] and dJ/dela in dJ[2m+1];
 * the call synchronises the stream. work[m] has lam[m]'s layout (that of members[m].H) and is
 * overwritten. members and params must be those of the taped run: the tape's header holds a
 * hash of their layouts and parameters. The arithmetic per member is that of
 * cg_sia_adjoint_run. */
CG_API int cg_sia_ensemble_adjoint_run(cg_ctx* ctx, int nmembers, const cg_sia_member* members,
                                       const cg_sia_params* params, const void* tape, size_t tape_bytes,
                                       const cg_field* lam, const cg_field* work, double* dJ);

/* Reverse step of the SIA time loop of cg_sia_run (no reference counterpart: the reference has
 * no adjoint). H is the state H_n at the start of the forward step, with the ghost layer the
 * forward step read (bc! Neumann copies after every step). lam holds dJ/dH_{n+1} at the
 * interior cells. The entry writes dJ/dH_n at the interior cells into lam_out (the ghost
 * cells' terms folded into the cells they copy). The step's dJ/dGamma and dJ/dela accumulate
 * on the device: a call with dJ == NULL only adds to them, and a call with dJ (host memory)
 * adds the accumulated sums to dJ[0] (Gamma) and dJ[1] (ela), starts them again from zero and
 * synchronises the stream. The step's quantities (D, its maximum and dt, the fluxes, the masks
 * of max(H, 0) and of the mass balance's cap) are recomputed from H with the forward's
 * arithmetic. The adaptive dt is differentiated through max D at the cell attaining it when
 * dt is below dt_max. The kernels replay from one CUDA graph per argument set. */
CG_API int cg_sia_adjoint_step(cg_ctx* ctx, const cg_grid* grid, const cg_field* H, const cg_field* B,
                               const cg_sia_params* p, const cg_field* lam, const cg_field* lam_out,
                               double* dJ);

/* Bytes of a tape that records `nsteps` steps of cg_sia_run_taped for an H of this layout:
 * a 256-byte header, then per step 256 bytes of words and 9 arrays of H's allocation. No
 * context and no device work. */
CG_API int cg_sia_tape_bytes(const cg_grid* grid, const cg_field* H, int nsteps, size_t* bytes);

/* cg_sia_run (same arguments, same results bit for bit) that also records, for each of its
 * `nsteps` (>= 1) steps, what the reverse step needs: D, the face gradients, the derivatives
 * of D, W = -divg(q) + M, the two masks, and the step's Dmax, argmax and dt. `tape` is device
 * memory of at least cg_sia_tape_bytes bytes, 256-byte aligned (no reference counterpart). */
CG_API int cg_sia_run_taped(cg_ctx* ctx, const cg_grid* grid, const cg_field* H, const cg_field* B,
                            const cg_field* q, const cg_sia_params* p, int nsteps, void* tape,
                            size_t tape_bytes, double* t_host);

/* The reverse sweep over a tape of cg_sia_run_taped, in one call: on entry lam holds dJ/dH at
 * the interior cells after the taped run's last step; on return it holds dJ/dH at its start.
 * dJ (host, may be NULL) gains dJ/dGamma in dJ[0] and dJ/dela in dJ[1]; the call synchronises
 * the stream. `work` is a field of lam's layout, overwritten. lam, work and p must match the
 * taped run's layout and parameters (the tape's header is checked). The sweep reads the
 * tape and recomputes nothing; its arithmetic is that of cg_sia_adjoint_step. */
CG_API int cg_sia_adjoint_run(cg_ctx* ctx, const cg_grid* grid, const cg_sia_params* p, const void* tape,
                              size_t tape_bytes, const cg_field* lam, const cg_field* work, double* dJ);

#ifdef __cplusplus
}
#endif

#endif /* CHMY_GB300_H */
