/*
 * chmy_oracle.cpp — CPU restatement of Chmy.jl's staggered-grid hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the parity oracle: it is loaded by tests/,
 * by __graft_entry__.smoke() as the checker and by bench.py for the CPU-baseline leg.
 * The product (libchmy_gb300.so) never links or calls it.
 *
 * Every function restates the reference's arithmetic in the reference's operation order;
 * Julia `muladd` sites use std::fma (Julia lowers muladd to FMA on FMA-capable CPUs) and
 * everything else is compiled with -ffp-contract=off. Index ranges follow Chmy's Launcher:
 * kernels run over I in [0, n+1]^N (src/KernelLaunch.jl:41,109) where n = grid cells.
 *
 * Parity pin: the grid, field-layout, operator, interpolation and boundary-condition
 * pieces are checked against the known answers of the reference's own test-suite
 * (test/test_grids.jl, test_fields.jl, test_grid_operators.jl, test_interpolations.jl,
 * test_boundary_conditions.jl) by tests/test_oracle_kat.py. The solver kernels (the
 * examples) have no reference golden vectors (no reference test runs them): they are
 * pinned by that restated operator layer plus physics self-checks.
 */
#include "../include/chmy_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* Field view: element at logical index I is p[off + sum I_d * s_d] (src/Fields/field.jl:18). */
template <class T>
struct Fd {
    T* p = nullptr;
    int nd = 0;
    int n[3] = {1, 1, 1};
    int loc[3] = {0, 0, 0};
    long off = 0;
    long s[3] = {0, 0, 0};
    Fd() = default;
    explicit Fd(const cg_field& f) {
        p = static_cast<T*>(f.data);
        nd = f.ndim;
        for (int d = 0; d < 3; ++d) {
            n[d] = d < nd ? f.n[d] : 1;
            loc[d] = d < nd ? f.loc[d] : 0;
            s[d] = d < nd ? (long)f.stride[d] : 0;
            if (d < nd) off += (long)(2 * f.halo[d] - 1) * s[d];
        }
    }
    bool ok() const { return p != nullptr; }
    T& at(const int* I) const { return p[off + I[0] * s[0] + I[1] * s[1] + I[2] * s[2]]; }
    T& operator()(int i, int j, int k) const { return p[off + i * s[0] + j * s[1] + k * s[2]]; }
};

struct Gd {
    int nd;
    int n[3];
};

template <class T>
struct GridT {
    int nd;
    int n[3];
    T dx[3];
    T idx[3];
    explicit GridT(const cg_grid& g) {
        nd = g.ndim;
        for (int d = 0; d < 3; ++d) {
            n[d] = d < nd ? g.n[d] : 1;
            dx[d] = (T)g.spacing[d];
            idx[d] = (T)g.inv_spacing[d];
        }
    }
};

/* Loop over the Launcher range [0, n+1] in used dims, {0} in unused ones. */
template <class G, class F>
void launch_range(const G& g, F&& fn) {
    const int e0 = g.n[0] + 1;
    const int e1 = g.nd > 1 ? g.n[1] + 1 : 0;
    const int e2 = g.nd > 2 ? g.n[2] + 1 : 0;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k <= e2; ++k)
        for (int j = 0; j <= e1; ++j)
            for (int i = 0; i <= e0; ++i) fn(i, j, k);
}

/* Loop over the interior-cell range [1, n]^N (sia.jl launches with ws = size(grid, Center())). */
template <class G, class F>
void cell_range(const G& g, F&& fn) {
    const int e0 = g.n[0];
    const int e1 = g.nd > 1 ? g.n[1] : 0;
    const int e2 = g.nd > 2 ? g.n[2] : 0;
    const int b1 = g.nd > 1 ? 1 : 0;
    const int b2 = g.nd > 2 ? 1 : 0;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = b2; k <= e2; ++k)
        for (int j = b1; j <= e1; ++j)
            for (int i = 1; i <= e0; ++i) fn(i, j, k);
}

/* ---- operators (src/GridOperators/GridOperators.jl:23-38, partial_derivatives.jl) ---- */

/* left/right of a field evaluated from flipped(loc, dim): a Vertex field seen from a
 * Center point has (I, I+1); a Center field seen from a Vertex point has (I-1, I). */
template <class T>
inline T left(const Fd<T>& f, int d, int i, int j, int k) {
    int I[3] = {i, j, k};
    if (f.loc[d] == CG_CENTER) I[d] -= 1;
    return f.at(I);
}
template <class T>
inline T right(const Fd<T>& f, int d, int i, int j, int k) {
    int I[3] = {i, j, k};
    if (f.loc[d] == CG_VERTEX) I[d] += 1;
    return f.at(I);
}
/* δ = right - left; ∂ = δ * iΔ (multiply by the inverse spacing, partial_derivatives.jl:2-5). */
template <class T>
inline T delta(const Fd<T>& f, int d, int i, int j, int k) {
    return right(f, d, i, j, k) - left(f, d, i, j, k);
}
template <class T>
inline T partial(const Fd<T>& f, const GridT<T>& g, int d, int i, int j, int k) {
    return delta(f, d, i, j, k) * g.idx[d];
}

/* itp(f, to, rule) (src/GridOperators/interpolation.jl:14-56,225-229,262-278): weights 0.5 on
 * uniform axes; knots split on the LAST differing dimension first, so the first differing
 * dimension is interpolated innermost. rule 0 = Linear muladd(t, b-a, a); 1 = Harmonic. */
template <class T>
T itp_rec(const Fd<T>& f, const int* to, const int* dims, int m, const int* I, int rule) {
    if (m == 0) return f.at(I);
    const int d = dims[m - 1];
    int Il[3] = {I[0], I[1], I[2]}, Ir[3] = {I[0], I[1], I[2]};
    /* il(loc=from_d, from=to_d): il(Vertex, Center) = I, il(Center, Vertex) = I-1;
       ir(Vertex, Center) = I+1, ir(Center, Vertex) = I. */
    if (f.loc[d] == CG_VERTEX) {
        Ir[d] += 1;
    } else {
        Il[d] -= 1;
    }
    (void)to;
    const T a = itp_rec(f, to, dims, m - 1, Il, rule);
    const T b = itp_rec(f, to, dims, m - 1, Ir, rule);
    const T t = T(0.5);
    using std::fma;  // unqualified below: the dual type's overload is found by ADL
    if (rule == 0) return fma(t, b - a, a);
    const T ia = T(1) / a, ib = T(1) / b;
    return T(1) / fma(t, ib - ia, ia);
}
template <class T>
T itp(const Fd<T>& f, const int* to, int i, int j, int k, int rule) {
    int dims[3], m = 0;
    for (int d = 0; d < f.nd; ++d)
        if (f.loc[d] != to[d]) dims[m++] = d;
    const int I[3] = {i, j, k};
    return itp_rec(f, to, dims, m, I, rule);
}

/* divg(V) = Σ_d ∂(V_d) summed in dim order (field_operators.jl:121-126). */
template <class T>
inline T divg(const Fd<T>* V, const GridT<T>& g, int i, int j, int k) {
    T s = partial(V[0], g, 0, i, j, k);
    for (int d = 1; d < g.nd; ++d) s = s + partial(V[d], g, d, i, j, k);
    return s;
}

/* ∂(f, grid, dim, I) for the field-level entry (from = flipped(loc(f), dim)). */
template <class T>
inline T partial_at(const Fd<T>& f, const GridT<T>& g, int d, const int* I) {
    return partial(f, g, d, I[0], I[1], I[2]);
}

/* ∂²(f, dim, I) for f at its own location (partial_derivatives.jl:7-12). */
template <class T>
T partial2(const Fd<T>& f, const GridT<T>& g, int d, int i, int j, int k) {
    /* floc = flipped(loc, d); Ir = ir(floc_d, loc_d), Il = il(floc_d, loc_d). */
    int Il[3] = {i, j, k}, Ir[3] = {i, j, k};
    if (f.loc[d] == CG_CENTER) {
        Ir[d] += 1; /* ir(Vertex from Center) = I+1, il(Vertex from Center) = I */
    } else {
        Il[d] -= 1; /* ir(Center from Vertex) = I, il(Center from Vertex) = I-1 */
    }
    return (partial_at(f, g, d, Ir) - partial_at(f, g, d, Il)) * g.idx[d];
}

/* ∂k∂(f, k, dim, I) (partial_derivatives.jl:14-21): lerp(k, floc) * ∂f at the two fluxes. */
template <class T>
T partial_k_partial(const Fd<T>& f, const Fd<T>& kk, const GridT<T>& g, int d, int i, int j,
                    int k) {
    int Il[3] = {i, j, k}, Ir[3] = {i, j, k};
    if (f.loc[d] == CG_CENTER) {
        Ir[d] += 1;
    } else {
        Il[d] -= 1;
    }
    int floc[3] = {f.loc[0], f.loc[1], f.loc[2]};
    floc[d] = 1 - floc[d];
    const T kr = itp(kk, floc, Ir[0], Ir[1], Ir[2], 0);
    const T kl = itp(kk, floc, Il[0], Il[1], Il[2], 0);
    return (kr * partial_at(f, g, d, Ir) - kl * partial_at(f, g, d, Il)) * g.idx[d];
}

/* ---- boundary conditions (first_order_boundary_condition.jl:34-84, batch.jl:104-268) -- */

/* Phase (dim d, side s) of one field, applied literally over tangential indices 0..n_t+2
 * (worksize remove_dim(dim, size(grid, Vertex()) .+ 2), index J-1, batch.jl:243,265). */
template <class T>
void bc_phase(const Gd& g, const Fd<T>& f, const cg_bc& bc, int d, int s, T spacing_d) {
    using std::fma;
    const int kind = bc.kind[d][s];
    if (kind == CG_BC_NONE) return;
    const int ext = f.n[d]; /* firstindex = 1, lastindex = ext */
    int tdims[2], nt = 0;
    for (int t = 0; t < g.nd; ++t)
        if (t != d) tdims[nt++] = t;
    const int e0 = nt > 0 ? g.n[tdims[0]] + 2 : 0;
    const int e1 = nt > 1 ? g.n[tdims[1]] + 2 : 0;
    /* the value: bc.value[remove_dim(dim, I)...] for per-point values
       (first_order_boundary_condition.jl:38-40), else the constant */
    const T* vals = static_cast<const T*>(bc.values[d][s]);
    for (int b = 0; b <= e1; ++b)
        for (int a = 0; a <= e0; ++a) {
            const T val = vals ? vals[a + (long)b * (e0 + 1)] : (T)bc.value[d][s];
            int I[3] = {0, 0, 0};
            if (nt > 0) I[tdims[0]] = a;
            if (nt > 1) I[tdims[1]] = b;
            if (kind == CG_BC_PERIODIC) {
                /* ghost <- periodic image: Center 0 <- n, n+1 <- 1; Vertex 0 <- n, n+1 <- 1,
                   n+2 <- 2 (node n+1 is node 1). */
                const int n = g.n[d];
                if (s == 0) {
                    int Is[3] = {I[0], I[1], I[2]};
                    I[d] = 0;
                    Is[d] = n;
                    f.at(I) = f.at(Is);
                } else {
                    int Is[3] = {I[0], I[1], I[2]};
                    I[d] = n + 1;
                    Is[d] = 1;
                    f.at(I) = f.at(Is);
                    if (f.loc[d] == CG_VERTEX) {
                        I[d] = n + 2;
                        Is[d] = 2;
                        f.at(I) = f.at(Is);
                    }
                }
                continue;
            }
            if (kind == CG_BC_DIRICHLET && f.loc[d] == CG_VERTEX) {
                I[d] = s == 0 ? 1 : ext; /* halo_index: the boundary node itself */
                f.at(I) = val;
                continue;
            }
            const int gi = s == 0 ? 0 : ext + 1;  /* itp_halo_index */
            const int ni = s == 0 ? 1 : ext;      /* neighbor_index */
            int In[3] = {I[0], I[1], I[2]};
            I[d] = gi;
            In[d] = ni;
            const T b0 = f.at(In);
            if (kind == CG_BC_DIRICHLET) {
                /* Center: muladd(t, a - b, b), t = 2 on a UniformGrid */
                f.at(I) = fma(T(2), val - b0, b0);
            } else {
                /* Neumann: muladd(h, ±q, f[in]), minus on Side(1) */
                const T qs = s == 0 ? -val : val;
                f.at(I) = fma(spacing_d, qs, b0);
            }
        }
}

template <class T>
int bc_apply_t(const cg_grid* grid, int nfields, const cg_field* fields, const cg_bc* bcs) {
    Gd g{grid->ndim, {grid->n[0], grid->ndim > 1 ? grid->n[1] : 1, grid->ndim > 2 ? grid->n[2] : 1}};
    /* batch.jl:104-113: Dim N -> 1, Side(1) then Side(2); within a side, fields in order. */
    for (int d = g.nd - 1; d >= 0; --d)
        for (int s = 0; s < 2; ++s)
            for (int fi = 0; fi < nfields; ++fi) {
                Fd<T> f(fields[fi]);
                bc_phase(g, f, bcs[fi], d, s, (T)grid->spacing[d]);
            }
    return CG_OK;
}

/* ---- masked operators (src/GridOperators/masked_operators.jl:11-39) --------------------
 * Every operand value is multiplied by the mask at the operand's location and index:
 * left(f, ω) = f[Il] at(ω, loc(f), Il), right likewise, δ = right - left, ∂ = δ iΔ. The mask
 * is one weight field per location, indexed by the location's bits (Vertex along d = bit d). */
struct Mask {
    const cg_mask* m;
    template <class T>
    T at(const Fd<T>& f, const int* I) const {
        int bits = 0;
        for (int d = 0; d < 3; ++d)
            if (f.loc[d] == CG_VERTEX) bits |= 1 << d;
        return Fd<T>(m->at[bits]).at(I);
    }
};
template <class T>
inline T mleft(const Fd<T>& f, const Mask& w, int d, int i, int j, int k) {
    int I[3] = {i, j, k};
    if (f.loc[d] == CG_CENTER) I[d] -= 1;
    return f.at(I) * w.at(f, I);
}
template <class T>
inline T mright(const Fd<T>& f, const Mask& w, int d, int i, int j, int k) {
    int I[3] = {i, j, k};
    if (f.loc[d] == CG_VERTEX) I[d] += 1;
    return f.at(I) * w.at(f, I);
}
template <class T>
inline T mpartial(const Fd<T>& f, const Mask& w, const GridT<T>& g, int d, int i, int j, int k) {
    return (mright(f, w, d, i, j, k) - mleft(f, w, d, i, j, k)) * g.idx[d];
}
/* divg(V, ω, grid, I) = Σ_d ∂(V_d, ω, grid, d, I) in dim order (masked_field_operators.jl:52-57) */
template <class T>
inline T mdivg(const Fd<T>* V, const Mask& w, const GridT<T>& g, int i, int j, int k) {
    T s = mpartial(V[0], w, g, 0, i, j, k);
    for (int d = 1; d < g.nd; ++d) s = s + mpartial(V[d], w, g, d, i, j, k);
    return s;
}

/* ---- explicit diffusion (examples/diffusion_2d.jl:8-19) ---------------------------- */

template <class T>
void diffusion_compute_q_t(const cg_grid* grid, const cg_field* q, const cg_field* C, double chi) {
    GridT<T> g(*grid);
    Fd<T> c(*C);
    Fd<T> Q[3];
    for (int d = 0; d < g.nd; ++d) Q[d] = Fd<T>(q[d]);
    const T mchi = -(T)chi;
    launch_range(g, [&](int i, int j, int k) {
        for (int d = 0; d < g.nd; ++d) Q[d](i, j, k) = mchi * partial(c, g, d, i, j, k);
    });
}

template <class T>
void diffusion_update_C_t(const cg_grid* grid, const cg_field* C, const cg_field* q, double dt) {
    GridT<T> g(*grid);
    Fd<T> c(*C);
    Fd<T> Q[3];
    for (int d = 0; d < g.nd; ++d) Q[d] = Fd<T>(q[d]);
    const T Dt = (T)dt;
    launch_range(g, [&](int i, int j, int k) { c(i, j, k) = c(i, j, k) - Dt * divg(Q, g, i, j, k); });
}

/* the same kernels with the masked operators: q.d = -χ ∂d(C, ω), C -= dt divg(q, ω) */
template <class T>
void diffusion_compute_q_masked_t(const cg_grid* grid, const cg_field* q, const cg_field* C, double chi,
                                  const cg_mask* m) {
    GridT<T> g(*grid);
    Fd<T> c(*C);
    Fd<T> Q[3];
    for (int d = 0; d < g.nd; ++d) Q[d] = Fd<T>(q[d]);
    const Mask w{m};
    const T mchi = -(T)chi;
    launch_range(g, [&](int i, int j, int k) {
        for (int d = 0; d < g.nd; ++d) Q[d](i, j, k) = mchi * mpartial(c, w, g, d, i, j, k);
    });
}

template <class T>
void diffusion_update_C_masked_t(const cg_grid* grid, const cg_field* C, const cg_field* q, double dt,
                                 const cg_mask* m) {
    GridT<T> g(*grid);
    Fd<T> c(*C);
    Fd<T> Q[3];
    for (int d = 0; d < g.nd; ++d) Q[d] = Fd<T>(q[d]);
    const Mask w{m};
    const T Dt = (T)dt;
    launch_range(g, [&](int i, int j, int k) { c(i, j, k) = c(i, j, k) - Dt * mdivg(Q, w, g, i, j, k); });
}

/* ---- VE Stokes (examples/stokes_{2,3}d_inc_ve_T.jl) -------------------------------- */

struct Tens {
    int xx, yy, zz, xy, xz, yz;
};
inline Tens tens_index(int nd) {
    if (nd == 2) return Tens{0, 1, -1, 2, -1, -1};
    return Tens{0, 1, 2, 3, 4, 5};
}

template <class T>
void stokes_update_old_t(const cg_grid* grid, const cg_stokes_fields* f) {
    GridT<T> g(*grid);
    const int nt = g.nd == 2 ? 3 : 6;
    Fd<T> tau[6], tau_old[6];
    for (int c = 0; c < nt; ++c) {
        tau[c] = Fd<T>(f->tau[c]);
        tau_old[c] = Fd<T>(f->tau_old[c]);
    }
    Fd<T> Tt(f->T), To(f->T_old);
    launch_range(g, [&](int i, int j, int k) {
        if (Tt.ok() && To.ok()) To(i, j, k) = Tt(i, j, k);
        for (int c = 0; c < nt; ++c) tau_old[c](i, j, k) = tau[c](i, j, k);
    });
}

/* Variable-viscosity extension (the examples have a scalar eta): with ieta = 1/eta (cell),
 * inv_Gdt = 1/(G dt), eta_ve = 1/(ieta + inv_Gdt); shear components use ieta interpolated
 * with Chmy's Linear rule (a harmonic average of eta); the velocity PT step uses
 * nu_dtau * (min(ieta_l, ieta_r) + inv_Gdt) = nu_dtau / max(eta_ve_l, eta_ve_r). */
template <class T>
struct InvEta {
    Fd<T> eta, ieta;
    bool var = false, have_inv = false;
    explicit InvEta(const cg_stokes_fields* f) : eta(f->eta), ieta(f->inv_eta) {
        var = eta.ok() || ieta.ok();
        have_inv = ieta.ok();
    }
    T at(int i, int j, int k) const { return have_inv ? ieta(i, j, k) : T(1) / eta(i, j, k); }
    T at(const int* I) const { return have_inv ? ieta.at(I) : T(1) / eta.at(I); }
};

/* With `mask`, every derivative is the masked operator (mpartial, mdivg): the Stokes kernels
 * written with a FieldMask ω as in docs/src/concepts/grid_operators.md ("Masking"). */
template <class T>
void stokes_update_stress_t(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
                            const cg_mask* mask = nullptr) {
    GridT<T> g(*grid);
    const Mask w{mask};
    auto D = [&](const Fd<T>& fld, int d, int i, int j, int k) {
        return mask ? mpartial(fld, w, g, d, i, j, k) : partial(fld, g, d, i, j, k);
    };
    const int nd = g.nd;
    const Tens ti = tens_index(nd);
    Fd<T> V[3], tau[6], tau_old[6];
    for (int d = 0; d < nd; ++d) V[d] = Fd<T>(f->V[d]);
    const int nt = nd == 2 ? 3 : 6;
    for (int c = 0; c < nt; ++c) {
        tau[c] = Fd<T>(f->tau[c]);
        tau_old[c] = Fd<T>(f->tau_old[c]);
    }
    Fd<T> P(f->P), divV(f->divV);
    const InvEta<T> ie(f);
    const T G = (T)p->G, dt = (T)p->dt, dtau_Pr = (T)p->dtau_Pr, dtau_r = (T)p->dtau_r;
    const T eta_s = (T)p->eta, eta_ve_s = (T)p->eta_ve;
    const T inv_Gdt = T(1) / (G * dt), third = T(1) / T(3);
    launch_range(g, [&](int i, int j, int k) {
        const T exx = D(V[0], 0, i, j, k);
        const T eyy = D(V[1], 1, i, j, k);
        const T dv = mask ? mdivg(V, w, g, i, j, k) : divg(V, g, i, j, k);
        T dvm = dv;
        if (divV.ok()) {
            divV(i, j, k) = dv;
            dvm = divV(i, j, k);
        }
        T ieta_c = 0, eve_c = eta_ve_s;
        if (ie.var) {
            ieta_c = ie.at(i, j, k);
            eve_c = T(1) / (ieta_c + inv_Gdt);
        }
        P(i, j, k) = P(i, j, k) - dvm * eve_c * dtau_Pr;
        auto upd_diag = [&](int c, T edd) {
            const T t = tau[c](i, j, k), to_ = tau_old[c](i, j, k);
            T r;
            if (ie.var)
                r = -(t - to_) * inv_Gdt - t * ieta_c + T(2.0) * (edd - dvm * third);
            else  /* examples/stokes_2d_inc_ve_T.jl:28-29 */
                r = -(t - to_) / (G * dt) - t / eta_s + T(2.0) * (edd - dvm / T(3.0));
            tau[c](i, j, k) = t + r * eve_c * dtau_r;
        };
        auto upd_off = [&](int c, T eod, int a, int b) {
            const T t = tau[c](i, j, k), to_ = tau_old[c](i, j, k);
            if (ie.var) {
                /* ieta at the (a, b) edge: Linear rule over the 4 cells, dim a innermost */
                int I00[3] = {i, j, k}, I10[3] = {i, j, k}, I01[3] = {i, j, k}, I11[3] = {i, j, k};
                I00[a] -= 1; I00[b] -= 1;
                I10[b] -= 1;
                I01[a] -= 1;
                const T e00 = ie.at(I00), e10 = ie.at(I10), e01 = ie.at(I01), e11 = ie.at(I11);
                using std::fma;
                const T lo = fma(T(0.5), e10 - e00, e00);
                const T hi = fma(T(0.5), e11 - e01, e01);
                const T iev = fma(T(0.5), hi - lo, lo);
                const T eve = T(1) / (iev + inv_Gdt);
                const T r = -(t - to_) * inv_Gdt - t * iev + T(2.0) * eod;
                tau[c](i, j, k) = t + r * eve * dtau_r;
            } else {  /* examples/stokes_2d_inc_ve_T.jl:30 */
                const T r = -(t - to_) / (G * dt) - t / eta_s + T(2.0) * eod;
                tau[c](i, j, k) = t + r * eta_ve_s * dtau_r;
            }
        };
        if (nd == 2) {
            const T exy = T(0.5) * (D(V[0], 1, i, j, k) + D(V[1], 0, i, j, k));
            upd_diag(ti.xx, exx);
            upd_diag(ti.yy, eyy);
            upd_off(ti.xy, exy, 0, 1);
        } else {
            const T ezz = D(V[2], 2, i, j, k);
            const T exy = T(0.5) * (D(V[0], 1, i, j, k) + D(V[1], 0, i, j, k));
            const T exz = T(0.5) * (D(V[0], 2, i, j, k) + D(V[2], 0, i, j, k));
            const T eyz = T(0.5) * (D(V[1], 2, i, j, k) + D(V[2], 1, i, j, k));
            upd_diag(ti.xx, exx);
            upd_diag(ti.yy, eyy);
            upd_diag(ti.zz, ezz);
            upd_off(ti.xy, exy, 0, 1);
            upd_off(ti.xz, exz, 0, 2);
            upd_off(ti.yz, eyz, 1, 2);
        }
    });
}

template <class T>
void stokes_update_velocity_t(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
                              const cg_mask* mask = nullptr) {
    GridT<T> g(*grid);
    const Mask w{mask};
    auto D = [&](const Fd<T>& fld, int d, int i, int j, int k) {
        return mask ? mpartial(fld, w, g, d, i, j, k) : partial(fld, g, d, i, j, k);
    };
    const int nd = g.nd;
    const Tens ti = tens_index(nd);
    Fd<T> V[3], rV[3], rho[3], tau[6];
    for (int d = 0; d < nd; ++d) {
        V[d] = Fd<T>(f->V[d]);
        rV[d] = Fd<T>(f->r_V[d]);
        rho[d] = Fd<T>(f->rho_g[d]);
    }
    const int nt = nd == 2 ? 3 : 6;
    for (int c = 0; c < nt; ++c) tau[c] = Fd<T>(f->tau[c]);
    Fd<T> P(f->P);
    const InvEta<T> ie(f);
    const T G = (T)p->G, dt = (T)p->dt, nu_dtau = (T)p->nu_dtau, eta_ve_s = (T)p->eta_ve;
    const T inv_Gdt = T(1) / (G * dt);
    /* tensor component coupling momentum d with dimension e */
    auto comp = [&](int d, int e) -> int {
        if (d == e) return d == 0 ? ti.xx : (d == 1 ? ti.yy : ti.zz);
        const int a = std::min(d, e), b = std::max(d, e);
        if (a == 0 && b == 1) return ti.xy;
        if (a == 0 && b == 2) return ti.xz;
        return ti.yz;
    };
    launch_range(g, [&](int i, int j, int k) {
        for (int d = 0; d < nd; ++d) {
            /* r_V.d = -∂d(P) + ∂d(τ_dd) + Σ_{e≠d} ∂e(τ_de) [- ρg_d], summed left to right in
               the examples' order: x: (xx, xy, xz); y: (yy, xy, yz); z: (zz, xz, yz). */
            T r = -D(P, d, i, j, k) + D(tau[comp(d, d)], d, i, j, k);
            for (int e = 0; e < nd; ++e) {
                if (e == d) continue;
                r = r + D(tau[comp(d, e)], e, i, j, k);
            }
            if (rho[d].ok()) r = r - rho[d](i, j, k);
            T rv = r;
            if (rV[d].ok()) {
                rV[d](i, j, k) = r;
                rv = rV[d](i, j, k);
            }
            if (ie.var) {
                int Il[3] = {i, j, k};
                Il[d] -= 1;
                const T m = std::min(ie.at(Il), ie.at(i, j, k));
                V[d](i, j, k) = V[d](i, j, k) + rv * (nu_dtau * (m + inv_Gdt));
            } else {  /* examples/stokes_2d_inc_ve_T.jl:41-42 */
                V[d](i, j, k) = V[d](i, j, k) + rv * nu_dtau / eta_ve_s;
            }
        }
    });
}

template <class T>
void stokes_update_thermal_flux_t(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p) {
    GridT<T> g(*grid);
    const int nd = g.nd;
    Fd<T> V[3], qT[3];
    for (int d = 0; d < nd; ++d) {
        V[d] = Fd<T>(f->V[d]);
        qT[d] = Fd<T>(f->qT[d]);
    }
    Fd<T> Tt(f->T);
    const T lam = (T)p->lambda_rhoCp;
    launch_range(g, [&](int i, int j, int k) {
        for (int d = 0; d < nd; ++d) {
            /* T is Center: leftd(T, I) = T[I - e_d], rightd(T, I) = T[I] */
            const T v = V[d](i, j, k);
            qT[d](i, j, k) = -lam * partial(Tt, g, d, i, j, k) + std::max(v, T(0.0)) * left(Tt, d, i, j, k) +
                             std::min(v, T(0.0)) * right(Tt, d, i, j, k);
        }
    });
}

template <class T>
void stokes_update_thermal_t(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p) {
    GridT<T> g(*grid);
    Fd<T> qT[3];
    for (int d = 0; d < g.nd; ++d) qT[d] = Fd<T>(f->qT[d]);
    Fd<T> Tt(f->T), To(f->T_old);
    const T dt = (T)p->dt;
    launch_range(g, [&](int i, int j, int k) { Tt(i, j, k) = To(i, j, k) - dt * divg(qT, g, i, j, k); });
}

/* ---- reductions ------------------------------------------------------------------- */

template <class T>
double maxabs_t(const cg_field& fd, int* nonfinite) {
    Fd<T> f(fd);
    double m = 0.0;
    int bad = 0;
    const int e1 = f.nd > 1 ? f.n[1] : 1, e2 = f.nd > 2 ? f.n[2] : 1;
    for (int k = 1; k <= e2; ++k)
        for (int j = 1; j <= e1; ++j)
            for (int i = 1; i <= f.n[0]; ++i) {
                const double v = std::fabs((double)f(i, f.nd > 1 ? j : 0, f.nd > 2 ? k : 0));
                if (!std::isfinite(v)) bad = 1;
                if (std::isnan(v)) m = v;
                else if (!std::isnan(m) && v > m) m = v;
            }
    if (bad) *nonfinite = 1;
    return m;
}

/* ---- operator test kernels (test/test_grid_operators.jl, test_interpolations.jl) ---- */

/* op 0 divg1!: V.d = ∂d(C) ; op 1 divg2!: C1 = Σ∂(V.d), C2 = divg(V) ;
 * op 2 lapl!: C1 = Σ∂²(C), C2 = lapl(C) ; op 3 divg_grad1!: V.d = lerp(χ, loc(V.d))·∂d(C) ;
 * op 4 divg_grad2!: C1 = Σ∂(V.d), C2 = divg_grad(C, χ) ; op 5 vmag: C1 = vmag(V) ;
 * op 6 lerp: C1 (at its own loc) = lerp(C, loc(C1)) over [1, n_C1]^N (set! discrete range) ;
 * op 7 hlerp: as 6 with the harmonic rule. */
template <class T>
void op_kernel_t(int op, const cg_grid* grid, const cg_field* C, const cg_field* C1, const cg_field* C2,
                 const cg_field* V, const cg_field* chi) {
    GridT<T> g(*grid);
    Fd<T> c, c1, c2, k, v[3];
    if (C) c = Fd<T>(*C);
    if (C1) c1 = Fd<T>(*C1);
    if (C2) c2 = Fd<T>(*C2);
    if (chi) k = Fd<T>(*chi);
    if (V)
        for (int d = 0; d < g.nd; ++d) v[d] = Fd<T>(V[d]);
    if (op == 6 || op == 7) {
        const int e1 = c1.nd > 1 ? c1.n[1] : 0, e2 = c1.nd > 2 ? c1.n[2] : 0;
        for (int kk = c1.nd > 2 ? 1 : 0; kk <= e2; ++kk)
            for (int j = c1.nd > 1 ? 1 : 0; j <= e1; ++j)
                for (int i = 1; i <= c1.n[0]; ++i) c1(i, j, kk) = itp(c, c1.loc, i, j, kk, op - 6);
        return;
    }
    launch_range(g, [&](int i, int j, int kk) {
        switch (op) {
            case 0:
                for (int d = 0; d < g.nd; ++d) v[d](i, j, kk) = partial(c, g, d, i, j, kk);
                break;
            case 1: {
                T s = partial(v[0], g, 0, i, j, kk);
                for (int d = 1; d < g.nd; ++d) s = s + partial(v[d], g, d, i, j, kk);
                c1(i, j, kk) = s;
                c2(i, j, kk) = divg(v, g, i, j, kk);
                break;
            }
            case 2: {
                T s = partial2(c, g, 0, i, j, kk);
                for (int d = 1; d < g.nd; ++d) s = s + partial2(c, g, d, i, j, kk);
                c1(i, j, kk) = s;
                T l = partial2(c, g, 0, i, j, kk);
                for (int d = 1; d < g.nd; ++d) l = l + partial2(c, g, d, i, j, kk);
                c2(i, j, kk) = l;
                break;
            }
            case 3:
                for (int d = 0; d < g.nd; ++d) v[d](i, j, kk) = itp(k, v[d].loc, i, j, kk, 0) * partial(c, g, d, i, j, kk);
                break;
            case 4: {
                T s = partial(v[0], g, 0, i, j, kk);
                for (int d = 1; d < g.nd; ++d) s = s + partial(v[d], g, d, i, j, kk);
                c1(i, j, kk) = s;
                T t = partial_k_partial(c, k, g, 0, i, j, kk);
                for (int d = 1; d < g.nd; ++d) t = t + partial_k_partial(c, k, g, d, i, j, kk);
                c2(i, j, kk) = t;
                break;
            }
            case 5: {
                const int to[3] = {CG_CENTER, CG_CENTER, CG_CENTER};
                T s = itp(v[0], to, i, j, kk, 0);
                s = s * s;
                for (int d = 1; d < g.nd; ++d) {
                    const T a = itp(v[d], to, i, j, kk, 0);
                    s = s + a * a;
                }
                c1(i, j, kk) = std::sqrt(s);
                break;
            }
            default:
                break;
        }
    });
}

/* ---- PT variable-coefficient diffusion (no reference example; restated from the PT pattern
 *      of examples/stokes_2d_inc_ve_T.jl and the ∂k∂ flux of partial_derivatives.jl:14-21) --- */

template <class T>
void ptdiff_update_q_t(const cg_grid* grid, const cg_ptdiff_fields* f, const cg_ptdiff_params* p) {
    GridT<T> g(*grid);
    Fd<T> C(f->C), D(f->D), q[3];
    for (int d = 0; d < g.nd; ++d) q[d] = Fd<T>(f->q[d]);
    const T om = (T)p->omega_q;
    launch_range(g, [&](int i, int j, int k) {
        for (int d = 0; d < g.nd; ++d) {
            /* lerp(D, face_d): D Center seen from the face -> cells I-e_d, I */
            int Il[3] = {i, j, k};
            Il[d] -= 1;
            const T dl = D.at(Il), dc = D(i, j, k);
            using std::fma;  // unqualified: the dual type's overload is found by ADL
            const T Df = fma(T(0.5), dc - dl, dl);
            const T gC = partial(C, g, d, i, j, k);
            const T qo = q[d](i, j, k);
            q[d](i, j, k) = qo + (-(Df * gC) - qo) * om;
        }
    });
}

template <class T>
void ptdiff_update_C_t(const cg_grid* grid, const cg_ptdiff_fields* f, const cg_ptdiff_params* p) {
    GridT<T> g(*grid);
    Fd<T> C(f->C), Co(f->C_old), R(f->R), q[3];
    for (int d = 0; d < g.nd; ++d) q[d] = Fd<T>(f->q[d]);
    const T inv_dt = T(1) / (T)p->dt, dtc = (T)p->dtau_C;
    launch_range(g, [&](int i, int j, int k) {
        const T c = C(i, j, k);
        const T r = -(c - Co(i, j, k)) * inv_dt - divg(q, g, i, j, k);
        if (R.ok()) R(i, j, k) = r;
        C(i, j, k) = c + r * dtc;
    });
}

/* ---- shallow ice (examples/sia.jl) --------------------------------------------------- */

/* x^m by repeated multiplication (the restatement of Julia's integer power). */
template <class T>
inline T ipow(T x, int m) {
    if (m <= 0) return T(1);
    T r = x;
    for (int k = 1; k < m; ++k) r = r * x;
    return r;
}

template <class T>
struct Sia {
    GridT<T> g;
    Fd<T> H, B;
    T Gamma, As, beta, ela, m_max;
    int n;
    Sia(const cg_grid* grid, const cg_field* Hf, const cg_field* Bf, const cg_sia_params* p)
        : g(*grid), H(*Hf), B(*Bf) {
        Gamma = (T)p->Gamma;
        As = (T)p->As;
        beta = (T)p->beta;
        ela = (T)p->ela;
        m_max = (T)p->m_max;
        n = p->n;
    }
    /* S = B + H (examples/sia.jl:38-41) */
    T S(int i, int j) const { return B(i, j, 0) + H(i, j, 0); }
    /* ∇S.x at vertex-x index i: ∂x(S) = (S[i] - S[i-1]) iΔx; ∇S.y likewise (:43-44) */
    T gx(int i, int j) const { return (S(i, j) - S(i - 1, j)) * g.idx[0]; }
    T gy(int i, int j) const { return (S(i, j) - S(i, j - 1)) * g.idx[1]; }
    /* vmag(∇S) at cell (i, j): sqrt(lerp(∇S.x → C)^2 + lerp(∇S.y → C)^2) (field_operators.jl:187-191) */
    T vmag(int i, int j) const {
        using std::fma;
        using std::sqrt;
        const T a0 = gx(i, j), a1 = gx(i + 1, j);
        const T ax = fma(T(0.5), a1 - a0, a0);
        const T b0 = gy(i, j), b1 = gy(i, j + 1);
        const T ay = fma(T(0.5), b1 - b0, b0);
        return sqrt(ax * ax + ay * ay);
    }
    /* D = (Gamma H^(n+2) + As H^n) vmag^(n-1) (:46-49) */
    T D(int i, int j) const {
        const T h = H(i, j, 0);
        return (Gamma * ipow(h, n + 2) + As * ipow(h, n)) * ipow(vmag(i, j), n - 1);
    }
    /* M = min(beta (S - ela), m_max) (:51-54) */
    T M(int i, int j) const { return std::min(beta * (S(i, j) - ela), m_max); }
};

/* update_q! and bc!(q) for a prepared Sia (its parameters may carry tangents); *dmax gets
   maximum(interior(D)), the first cell (j outer, i inner) attaining it */
template <class T>
void sia_update_q_body(const cg_grid* grid, const Sia<T>& s, const cg_field* q, T* dmax) {
    using std::fma;
    Fd<T> qx(q[0]), qy(q[1]);
    const int nx = s.g.n[0], ny = s.g.n[1];
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            const T dl = s.D(i - 1, j), dc = s.D(i, j), dd = s.D(i, j - 1);
            const T Dx = fma(T(0.5), dc - dl, dl);
            const T Dy = fma(T(0.5), dc - dd, dd);
            qx(i, j, 0) = -Dx * s.gx(i, j);
            qy(i, j, 0) = -Dy * s.gy(i, j);
        }
    if (dmax) {
        T m = T(0.0);
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) {
                const T d = s.D(i, j);
                if (m < d) m = d;
            }
        *dmax = m;
    }
    cg_bc b[2];
    std::memset(b, 0, sizeof(b));
    b[0].kind[0][0] = b[0].kind[0][1] = CG_BC_DIRICHLET;
    b[1].kind[1][0] = b[1].kind[1][1] = CG_BC_DIRICHLET;
    bc_apply_t<T>(grid, 2, q, b);
}

/* update_H! and bc!(H) for a prepared Sia, with a T-typed time step */
template <class T>
void sia_update_H_body(const cg_grid* grid, Sia<T>& s, const cg_field* Hf, const cg_field* q, T Dt) {
    Fd<T> Q[3] = {Fd<T>(q[0]), Fd<T>(q[1]), Fd<T>()};
    const int nx = s.g.n[0], ny = s.g.n[1];
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            const T h = s.H(i, j, 0);
            const T m = s.M(i, j);
            s.H(i, j, 0) = std::max(h + Dt * (-divg(Q, s.g, i, j, 0) + m), T(0.0));
        }
    cg_bc b;
    std::memset(&b, 0, sizeof(b));
    b.kind[0][0] = b.kind[0][1] = b.kind[1][0] = b.kind[1][1] = CG_BC_NEUMANN;
    bc_apply_t<T>(grid, 1, Hf, &b);
}

template <class T>
void sia_update_q_t(const cg_grid* grid, const cg_field* q, const cg_field* Hf, const cg_field* Bf,
                    const cg_sia_params* p, double* dmax) {
    Sia<T> s(grid, Hf, Bf, p);
    Fd<T> qx(q[0]), qy(q[1]);
    const int nx = s.g.n[0], ny = s.g.n[1];
    /* update_q! over ws = size(grid, Center()) = [1, n]^2 (:62-63,72) */
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            /* lerp(D, (Vertex, Center)): D Center seen from the x face -> cells i-1, i */
            const T dl = s.D(i - 1, j), dc = s.D(i, j), dd = s.D(i, j - 1);
            const T Dx = std::fma(T(0.5), dc - dl, dl);
            const T Dy = std::fma(T(0.5), dc - dd, dd);
            qx(i, j, 0) = -Dx * s.gx(i, j);
            qy(i, j, 0) = -Dy * s.gy(i, j);
        }
    if (dmax) {
        double m = 0;
        for (int j = 1; j <= ny; ++j)
            for (int i = 1; i <= nx; ++i) m = std::max(m, (double)s.D(i, j));
        *dmax = m;
    }
    /* bc!(arch, grid, q.x => (x = Dirichlet()), q.y => (y = Dirichlet())) (:73) */
    cg_bc b[2];
    std::memset(b, 0, sizeof(b));
    b[0].kind[0][0] = b[0].kind[0][1] = CG_BC_DIRICHLET;
    b[1].kind[1][0] = b[1].kind[1][1] = CG_BC_DIRICHLET;
    bc_apply_t<T>(grid, 2, q, b);
}

template <class T>
void sia_update_H_t(const cg_grid* grid, const cg_field* Hf, const cg_field* q, const cg_field* Bf, double dt,
                    const cg_sia_params* p) {
    Sia<T> s(grid, Hf, Bf, p);
    Fd<T> Q[3] = {Fd<T>(q[0]), Fd<T>(q[1]), Fd<T>()};
    const T Dt = (T)dt;
    const int nx = s.g.n[0], ny = s.g.n[1];
    /* M depends on S = B + H: evaluate it for all cells before H changes (the kernel reads
       H[I] and M[I] of the same cell only) */
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            const T h = s.H(i, j, 0);
            const T m = s.M(i, j);
            s.H(i, j, 0) = std::max(h + Dt * (-divg(Q, s.g, i, j, 0) + m), T(0.0));
        }
    cg_bc b;
    std::memset(&b, 0, sizeof(b));
    b.kind[0][0] = b.kind[0][1] = b.kind[1][0] = b.kind[1][1] = CG_BC_NEUMANN;
    bc_apply_t<T>(grid, 1, Hf, &b);
}

/* ---- forward-mode dual numbers: exact tangents of the restated loop ---------------------
 * A value and its derivatives along two directions; every operation is the value's own plus
 * its first-order rule. Comparisons (max, min, the kinks) act on the value. The restated SIA
 * step runs on it unchanged (its fma and sqrt calls are unqualified), so the tangents are the
 * derivatives of exactly the arithmetic above. */
struct Dual {
    double v = 0.0;
    double d[2] = {0.0, 0.0};
    Dual() = default;
    Dual(double x) : v(x) {}
    explicit operator double() const { return v; }
};
inline Dual operator+(const Dual& a, const Dual& b) {
    Dual r(a.v + b.v);
    for (int k = 0; k < 2; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
inline Dual operator-(const Dual& a, const Dual& b) {
    Dual r(a.v - b.v);
    for (int k = 0; k < 2; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
inline Dual operator-(const Dual& a) {
    Dual r(-a.v);
    for (int k = 0; k < 2; ++k) r.d[k] = -a.d[k];
    return r;
}
inline Dual operator*(const Dual& a, const Dual& b) {
    Dual r(a.v * b.v);
    for (int k = 0; k < 2; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
inline Dual operator/(const Dual& a, const Dual& b) {
    Dual r(a.v / b.v);
    for (int k = 0; k < 2; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
    return r;
}
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
inline Dual fma(const Dual& a, const Dual& b, const Dual& c) {
    Dual r(std::fma(a.v, b.v, c.v));
    for (int k = 0; k < 2; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k] + c.d[k];
    return r;
}
inline Dual sqrt(const Dual& a) {
    Dual r(std::sqrt(a.v));
    for (int k = 0; k < 2; ++k) r.d[k] = r.v > 0.0 ? a.d[k] / (2.0 * r.v) : 0.0;
    return r;
}

/* A field descriptor over `storage` with the layout of `like` (same strides and halo). */
template <class T>
cg_field like_field(const cg_field& like, std::vector<T>& storage) {
    long span = 1;
    for (int d = 0; d < like.ndim; ++d) span += (long)(like.n[d] + 4 * like.halo[d] - 1) * like.stride[d];
    storage.assign((size_t)span, T(0.0));
    cg_field f = like;
    f.data = storage.data();
    return f;
}

/* set!(f, grid, func) of a FunctionField (src/Fields/function_field.jl:49-59, Continuous form) for
   the function forms of cg_function, at every padded point: func(coord(grid, loc, I)...,
   parameters...) with coord of src/Grids/uniform_axis.jl (Vertex muladd(I-1, Δ, o), Center
   muladd(I-1, Δ, muladd(0.5, Δ, o))) in the field's precision. CG_FN_BALL is init_incl of
   examples/stokes_2d_inc_ve_T.jl:106: ifelse((x - x0)^2 + (y - y0)^2 < r^2, in, out). */
template <class T>
void function_fill_t(const cg_grid* grid, const cg_function* fn, const cg_field& fd) {
    Fd<T> f(fd);
    const int nd = fd.ndim;
    T p[8];
    for (int q = 0; q < 8; ++q) p[q] = (T)fn->p[q];
    auto coord = [&](int d, int I) {
        const T dx = (T)grid->spacing[d], o = (T)grid->origin[d];
        const T base = fd.loc[d] == CG_VERTEX ? o : std::fma(T(0.5), dx, o);
        return std::fma(T(I - 1), dx, base);
    };
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < nd; ++d) {
        lo[d] = 1 - 2 * fd.halo[d];
        hi[d] = fd.n[d] + 2 * fd.halo[d];
    }
    for (int k = lo[2]; k <= hi[2]; ++k)
        for (int j = lo[1]; j <= hi[1]; ++j)
            for (int i = lo[0]; i <= hi[0]; ++i) {
                const int I[3] = {i, j, k};
                T x[3] = {T(0), T(0), T(0)};
                for (int d = 0; d < nd; ++d) x[d] = coord(d, I[d]);
                T v = T(0);
                if (fn->kind == CG_FN_CONST) {
                    v = p[0];
                } else if (fn->kind == CG_FN_BALL) {
                    T r2 = (x[0] - p[0]) * (x[0] - p[0]);
                    for (int d = 1; d < nd; ++d) r2 = r2 + (x[d] - p[d]) * (x[d] - p[d]);
                    v = r2 < p[3] * p[3] ? p[4] : p[5];
                } else if (fn->kind == CG_FN_AFFINE) {
                    v = p[0];
                    for (int d = 0; d < nd; ++d) v = v + p[1 + d] * x[d];
                }
                f(i, nd > 1 ? j : 0, nd > 2 ? k : 0) = v;
            }
}

}  // namespace

/* ==== extern "C" surface (names mirror the library's cg_* entry points) =============== */
extern "C" {

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int or_bc_apply(const cg_grid* grid, int nfields, const cg_field* fields, const cg_bc* bcs) {
    if (nfields <= 0) return CG_OK;
    if (fields[0].dtype == CG_F64) return bc_apply_t<double>(grid, nfields, fields, bcs);
    return bc_apply_t<float>(grid, nfields, fields, bcs);
}

int or_maxabs(int nfields, const cg_field* fields, double* out, int32_t* nonfinite) {
    int bad = 0;
    for (int i = 0; i < nfields; ++i)
        out[i] = fields[i].dtype == CG_F64 ? maxabs_t<double>(fields[i], &bad) : maxabs_t<float>(fields[i], &bad);
    if (nonfinite) *nonfinite = bad;
    return CG_OK;
}

/* The PT iterations of the VE Stokes step with a viscosity field (update_stress!,
   update_velocity!, bc!(V => bc_V[d]) each; examples/stokes_2d_inc_ve_T.jl:20-43 with the
   variable-viscosity rules above) run in dual numbers until the value and both tangents reach
   their fixed point. The tangents are the exact derivatives of the converged discrete state
   with respect to log(eta) along the directions dir[0], dir[1] (FP64 fields of eta's layout;
   eta.d[k] = eta dir[k] at every point, so a direction that is zero outside the interior
   leaves the ghost viscosities fixed). `f` holds the FP64 initial state (V, r_V, P, divV, tau,
   tau_old and eta are required; inv_eta must be absent). Every `ncheck` iterations the
   residuals are read: max |r_V| over the points not fixed by bc_V (interior points, boundary
   nodes excluded) and max |divV| over the cells. Converged when the value's are <= tol and
   each tangent's are <= tol max(1, max |dV_k|). dV[k nd + d] (FP64, V[d]'s layout) receive
   the tangents of V[d]; the value stays in f. Returns 0 when converged within max_iter, else
   4 (timeout); *iterations gets the count. */
int or_stokes_solve_tangent(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
                            const cg_bc* bc_V, const cg_field* dir, double tol, int max_iter, int ncheck,
                            const cg_field* dV, int* iterations) {
    const int nd = grid->ndim, nt = nd == 2 ? 3 : 6;
    if (!f->eta.data || f->inv_eta.data || !f->divV.data || !f->P.data) return CG_ERR_ARG;
    std::vector<std::vector<Dual>> store;
    store.reserve(40);
    cg_stokes_fields fD;
    std::memset(&fD, 0, sizeof(fD));
    auto span_of = [](const cg_field& a) {
        long span = 1;
        for (int d = 0; d < a.ndim; ++d) span += (long)(a.n[d] + 4 * a.halo[d] - 1) * a.stride[d];
        return span;
    };
    auto dualize = [&](const cg_field& src, cg_field& dst) {
        if (!src.data) return;
        store.emplace_back();
        dst = like_field(src, store.back());
        const double* s = static_cast<const double*>(src.data);
        Dual* t = store.back().data();
        for (long q = 0; q < span_of(src); ++q) t[q] = Dual(s[q]);
    };
    for (int d = 0; d < nd; ++d) {
        dualize(f->V[d], fD.V[d]);
        dualize(f->r_V[d], fD.r_V[d]);
        dualize(f->rho_g[d], fD.rho_g[d]);
        if (!f->V[d].data || !f->r_V[d].data) return CG_ERR_ARG;
    }
    for (int c = 0; c < nt; ++c) {
        dualize(f->tau[c], fD.tau[c]);
        dualize(f->tau_old[c], fD.tau_old[c]);
        if (!f->tau[c].data || !f->tau_old[c].data) return CG_ERR_ARG;
    }
    dualize(f->P, fD.P);
    dualize(f->divV, fD.divV);
    dualize(f->eta, fD.eta);
    {
        Dual* e = static_cast<Dual*>(fD.eta.data);
        for (int k = 0; k < 2; ++k) {
            const double* w = static_cast<const double*>(dir[k].data);
            for (long q = 0; q < span_of(f->eta); ++q) e[q].d[k] = e[q].v * w[q];
        }
    }
    const int n0 = grid->n[0], n1 = nd > 1 ? grid->n[1] : 1, n2 = nd > 2 ? grid->n[2] : 1;
    auto residuals = [&](double* out /* value, tangent 0, tangent 1, max |dV_0|, max |dV_1| */) {
        for (int k = 0; k < 5; ++k) out[k] = 0.0;
        auto take = [&](const Dual& r) {
            out[0] = std::max(out[0], std::fabs(r.v));
            out[1] = std::max(out[1], std::fabs(r.d[0]));
            out[2] = std::max(out[2], std::fabs(r.d[1]));
        };
        for (int d = 0; d < nd; ++d) {
            Fd<Dual> r(fD.r_V[d]), v(fD.V[d]);
            for (int k = (nd > 2 ? 1 : 0); k <= (nd > 2 ? n2 : 0); ++k)
                for (int j = 1; j <= n1; ++j)
                    for (int i = 1; i <= n0; ++i) {
                        const int I[3] = {i, j, k};
                        if (I[d] == 1) continue;  // the boundary node of V[d] along d
                        take(r(i, j, k));
                        out[3] = std::max(out[3], std::fabs(v(i, j, k).d[0]));
                        out[4] = std::max(out[4], std::fabs(v(i, j, k).d[1]));
                    }
        }
        Fd<Dual> dv(fD.divV);
        for (int k = (nd > 2 ? 1 : 0); k <= (nd > 2 ? n2 : 0); ++k)
            for (int j = 1; j <= n1; ++j)
                for (int i = 1; i <= n0; ++i) take(dv(i, j, k));
    };
    bc_apply_t<Dual>(grid, nd, fD.V, bc_V);
    int it = 0;
    bool conv = false;
    while (it < max_iter && !conv) {
        for (int c = 0; c < ncheck && it < max_iter; ++c, ++it) {
            stokes_update_stress_t<Dual>(grid, &fD, p);
            stokes_update_velocity_t<Dual>(grid, &fD, p);
            bc_apply_t<Dual>(grid, nd, fD.V, bc_V);
        }
        double r[5];
        residuals(r);
        conv = r[0] <= tol && r[1] <= tol * std::max(1.0, r[3]) && r[2] <= tol * std::max(1.0, r[4]);
    }
    for (int d = 0; d < nd; ++d) {
        const Dual* v = static_cast<const Dual*>(fD.V[d].data);
        double* val = static_cast<double*>(f->V[d].data);
        for (long q = 0; q < span_of(f->V[d]); ++q) val[q] = v[q].v;
        for (int k = 0; k < 2; ++k) {
            double* o = static_cast<double*>(dV[k * nd + d].data);
            for (long q = 0; q < span_of(f->V[d]); ++q) o[q] = v[q].d[k];
        }
    }
    if (iterations) *iterations = it;
    return conv ? CG_OK : CG_ERR_TIMEOUT;
}

/* The time loop of cg_ptdiff_run (nsteps implicit steps: C_old <- C, then npt PT iterations
   of update_q, update_C and bc!(C => bc)) in dual numbers, with tangents along the two
   log-diffusivity directions dir[0], dir[1] (FP64, D's layout: D.d[k] = D dir[k] at every
   point). f holds FP64 host fields C, C_old, D and q (R must be absent); C advances in place.
   dC[k] (FP64, C's layout) receive the exact derivatives of the final C of this discrete loop
   (with its npt iterations per step) along dir[k]. */
int or_ptdiff_run_tangent(const cg_grid* grid, const cg_ptdiff_fields* f, const cg_ptdiff_params* p,
                          const cg_bc* bc, int nsteps, int npt, const cg_field* dir, const cg_field* dC) {
    const int nd = grid->ndim;
    if (!f->C.data || !f->C_old.data || !f->D.data || f->R.data) return CG_ERR_ARG;
    auto span_of = [](const cg_field& a) {
        long span = 1;
        for (int d = 0; d < a.ndim; ++d) span += (long)(a.n[d] + 4 * a.halo[d] - 1) * a.stride[d];
        return span;
    };
    std::vector<std::vector<Dual>> store;
    store.reserve(8);
    cg_ptdiff_fields fD;
    std::memset(&fD, 0, sizeof(fD));
    auto dualize = [&](const cg_field& src, cg_field& dst) {
        store.emplace_back();
        dst = like_field(src, store.back());
        const double* s = static_cast<const double*>(src.data);
        Dual* t = store.back().data();
        for (long q = 0; q < span_of(src); ++q) t[q] = Dual(s[q]);
    };
    dualize(f->C, fD.C);
    dualize(f->C_old, fD.C_old);
    dualize(f->D, fD.D);
    for (int d = 0; d < nd; ++d) {
        if (!f->q[d].data) return CG_ERR_ARG;
        dualize(f->q[d], fD.q[d]);
    }
    {
        Dual* e = static_cast<Dual*>(fD.D.data);
        for (int k = 0; k < 2; ++k) {
            const double* w = static_cast<const double*>(dir[k].data);
            for (long q = 0; q < span_of(f->D); ++q) e[q].d[k] = e[q].v * w[q];
        }
    }
    Dual* c = static_cast<Dual*>(fD.C.data);
    Dual* co = static_cast<Dual*>(fD.C_old.data);
    const long cspan = std::min(span_of(f->C), span_of(f->C_old));
    for (int step = 0; step < nsteps; ++step) {
        for (long q = 0; q < cspan; ++q) co[q] = c[q];
        for (int it = 0; it < npt; ++it) {
            ptdiff_update_q_t<Dual>(grid, &fD, p);
            ptdiff_update_C_t<Dual>(grid, &fD, p);
            bc_apply_t<Dual>(grid, 1, &fD.C, bc);
        }
    }
    double* cv = static_cast<double*>(f->C.data);
    for (long q = 0; q < span_of(f->C); ++q) cv[q] = c[q].v;
    for (int k = 0; k < 2; ++k) {
        double* o = static_cast<double*>(dC[k].data);
        for (long q = 0; q < span_of(f->C); ++q) o[q] = c[q].d[k];
    }
    return CG_OK;
}

/* The SIA time loop of examples/sia.jl:71-81 (update_q!, bc!, dt = min(Δ²/max D/cfl,
   dt_max), update_H!, bc!) in dual numbers: H (FP64) is advanced `nsteps` steps, and
   dH_dGamma, dH_dela (FP64, H's layout, zero on entry) receive the exact derivatives of the
   final H with respect to Gamma and ela. q (2 fields, FP64) is the loop's flux storage. */
int or_sia_run_tangent(const cg_grid* grid, const cg_field* H, const cg_field* B, const cg_field* q,
                       const cg_sia_params* p, int nsteps, const cg_field* dH_dGamma, const cg_field* dH_dela) {
    std::vector<Dual> hs, bs, q0s, q1s;
    const cg_field Hd = like_field(*H, hs), Bd = like_field(*B, bs);
    cg_field Qd[3] = {like_field(q[0], q0s), like_field(q[1], q1s), cg_field()};
    Fd<double> h(*H), b(*B);
    Fd<Dual> hD(Hd), bD(Bd);
    const int nx = grid->n[0], ny = grid->n[1];
    for (int j = -1; j <= ny + 2; ++j)
        for (int i = -1; i <= nx + 2; ++i) {
            hD(i, j, 0) = Dual(h(i, j, 0));
            bD(i, j, 0) = Dual(b(i, j, 0));
        }
    Sia<Dual> s(grid, &Hd, &Bd, p);
    s.Gamma.d[0] = 1.0;  // direction 0: Gamma
    s.ela.d[1] = 1.0;    // direction 1: ela
    const double dx = std::min(grid->spacing[0], grid->spacing[1]);
    for (int step = 0; step < nsteps; ++step) {
        Dual dmax;
        sia_update_q_body<Dual>(grid, s, Qd, &dmax);
        const Dual qdt = Dual(dx * dx) / dmax / Dual(p->cfl);
        const Dual dt = (dmax.v > 0.0 && qdt.v < p->dt_max) ? qdt : Dual(p->dt_max);
        sia_update_H_body<Dual>(grid, s, &Hd, Qd, dt);
    }
    Fd<double> gG(*dH_dGamma), gE(*dH_dela);
    for (int j = -1; j <= ny + 2; ++j)
        for (int i = -1; i <= nx + 2; ++i) {
            h(i, j, 0) = hD(i, j, 0).v;
            gG(i, j, 0) = hD(i, j, 0).d[0];
            gE(i, j, 0) = hD(i, j, 0).d[1];
        }
    return CG_OK;
}

/* The explicit diffusion loop of examples/diffusion_2d.jl:43-47 (compute_q!, update_C!, then
   bc!(C => bc)) in dual numbers, restated from the flux form of :8-19: tangent 0 along chi,
   tangent 1 along the initial-state direction `dir` (FP64, C's layout, read at every padded
   point; bc!(C) is applied once before the loop, so the ghost cells' tangents follow the
   interior's). C (FP64) advances `nsteps` steps in place; q (ndim FP64 face fields) is the loop's
   flux storage (the update reads its index n+2, which compute_q! never writes: keep it zero).
   dC[k] (FP64, C's layout) receive the exact derivatives of the final C along the two tangents. */
int or_diffusion_run_tangent(const cg_grid* grid, const cg_field* C, const cg_field* q, double chi, double dt,
                             const cg_bc* bc, int nsteps, const cg_field* dir, const cg_field* dC) {
    const int nd = grid->ndim;
    if (C->dtype != CG_F64 || dir->dtype != CG_F64) return CG_ERR_ARG;
    auto span_of = [](const cg_field& a) {
        long span = 1;
        for (int d = 0; d < a.ndim; ++d) span += (long)(a.n[d] + 4 * a.halo[d] - 1) * a.stride[d];
        return span;
    };
    std::vector<Dual> cs, qs[3];
    const cg_field Cd = like_field(*C, cs);
    cg_field Qd[3];
    for (int d = 0; d < nd; ++d) {
        if (!q[d].data || q[d].dtype != CG_F64) return CG_ERR_ARG;
        Qd[d] = like_field(q[d], qs[d]);
        const double* src = static_cast<const double*>(q[d].data);
        for (long e = 0; e < span_of(q[d]); ++e) qs[d][e] = Dual(src[e]);
    }
    {
        const double* c0 = static_cast<const double*>(C->data);
        const double* w = static_cast<const double*>(dir->data);
        for (long e = 0; e < span_of(*C); ++e) {
            cs[e] = Dual(c0[e]);
            cs[e].d[1] = w[e];
        }
    }
    bc_apply_t<Dual>(grid, 1, &Cd, bc);
    GridT<Dual> g(*grid);
    Fd<Dual> c(Cd);
    Fd<Dual> Q[3];
    for (int d = 0; d < nd; ++d) Q[d] = Fd<Dual>(Qd[d]);
    Dual chiD(chi);
    chiD.d[0] = 1.0;
    const Dual mchi = -chiD, Dt(dt);
    for (int step = 0; step < nsteps; ++step) {
        launch_range(g, [&](int i, int j, int k) {
            for (int d = 0; d < nd; ++d) Q[d](i, j, k) = mchi * partial(c, g, d, i, j, k);
        });
        launch_range(g, [&](int i, int j, int k) { c(i, j, k) = c(i, j, k) - Dt * divg(Q, g, i, j, k); });
        bc_apply_t<Dual>(grid, 1, &Cd, bc);
    }
    double* cv = static_cast<double*>(C->data);
    for (long e = 0; e < span_of(*C); ++e) cv[e] = cs[e].v;
    for (int k = 0; k < 2; ++k) {
        double* o = static_cast<double*>(dC[k].data);
        for (long e = 0; e < span_of(*C); ++e) o[e] = cs[e].d[k];
    }
    return CG_OK;
}

/* One thermal step of examples/stokes_2d_inc_ve_T.jl:45-60 (update_thermal_flux!,
   update_thermal!, then bc!(T => bc_T)) in dual numbers: tangent 0 along the directions dT,
   dT_old and dV[d] (FP64, in the layouts of T, T_old and V[d], read at every padded point; bc!(T)
   is applied to T first, so its ghost cells' tangents follow the interior), tangent 1 along
   lambda_rhoCp. f holds FP64 host fields T (the step's input; receives T_out), T_old, V and qT
   (flux storage, zero at the face index n+2 the flux kernel never writes). dTout[k] (FP64, T's
   layout) receive the tangents of T_out. */
int or_thermal_step_tangent(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
                            const cg_bc* bc_T, const cg_field* dT, const cg_field* dTold, const cg_field* dV,
                            const cg_field* dTout) {
    const int nd = grid->ndim;
    auto span_of = [](const cg_field& a) {
        long span = 1;
        for (int d = 0; d < a.ndim; ++d) span += (long)(a.n[d] + 4 * a.halo[d] - 1) * a.stride[d];
        return span;
    };
    std::vector<std::vector<Dual>> store;
    store.reserve(16);
    auto dualize = [&](const cg_field& src, const cg_field* dir) {
        store.emplace_back();
        cg_field dst = like_field(src, store.back());
        const double* s = static_cast<const double*>(src.data);
        const double* w = dir ? static_cast<const double*>(dir->data) : nullptr;
        Dual* t = store.back().data();
        for (long q = 0; q < span_of(src); ++q) {
            t[q] = Dual(s[q]);
            if (w) t[q].d[0] = w[q];
        }
        return dst;
    };
    if (f->T.dtype != CG_F64) return CG_ERR_ARG;
    const cg_field Td = dualize(f->T, dT), Tod = dualize(f->T_old, dTold);
    cg_field Vd[3], Qd[3];
    for (int d = 0; d < nd; ++d) {
        Vd[d] = dualize(f->V[d], &dV[d]);
        Qd[d] = dualize(f->qT[d], nullptr);
    }
    bc_apply_t<Dual>(grid, 1, &Td, bc_T);
    GridT<Dual> g(*grid);
    Fd<Dual> Tt(Td), To(Tod), V[3], qT[3];
    for (int d = 0; d < nd; ++d) {
        V[d] = Fd<Dual>(Vd[d]);
        qT[d] = Fd<Dual>(Qd[d]);
    }
    Dual lam(p->lambda_rhoCp);
    lam.d[1] = 1.0;
    const Dual dt(p->dt), zero(0.0);
    launch_range(g, [&](int i, int j, int k) {
        for (int d = 0; d < nd; ++d) {
            const Dual v = V[d](i, j, k);
            qT[d](i, j, k) = -lam * partial(Tt, g, d, i, j, k) + std::max(v, zero) * left(Tt, d, i, j, k) +
                             std::min(v, zero) * right(Tt, d, i, j, k);
        }
    });
    launch_range(g, [&](int i, int j, int k) { Tt(i, j, k) = To(i, j, k) - dt * divg(qT, g, i, j, k); });
    bc_apply_t<Dual>(grid, 1, &Td, bc_T);
    const Dual* tv = static_cast<const Dual*>(Td.data);
    double* out = static_cast<double*>(f->T.data);
    for (long q = 0; q < span_of(f->T); ++q) out[q] = tv[q].v;
    for (int k = 0; k < 2; ++k) {
        double* o = static_cast<double*>(dTout[k].data);
        for (long q = 0; q < span_of(f->T); ++q) o[q] = tv[q].d[k];
    }
    return CG_OK;
}

int or_function_fill(const cg_grid* grid, const cg_function* fn, const cg_field* f) {
    if (f->dtype == CG_F64) function_fill_t<double>(grid, fn, *f);
    else function_fill_t<float>(grid, fn, *f);
    return CG_OK;
}

int or_diffusion_compute_q(const cg_grid* grid, const cg_field* q, const cg_field* C, double chi) {
    if (C->dtype == CG_F64) diffusion_compute_q_t<double>(grid, q, C, chi);
    else diffusion_compute_q_t<float>(grid, q, C, chi);
    return CG_OK;
}

int or_diffusion_compute_q_masked(const cg_grid* grid, const cg_field* q, const cg_field* C, double chi,
                                  const cg_mask* m) {
    if (C->dtype == CG_F64) diffusion_compute_q_masked_t<double>(grid, q, C, chi, m);
    else diffusion_compute_q_masked_t<float>(grid, q, C, chi, m);
    return CG_OK;
}

int or_diffusion_update_C_masked(const cg_grid* grid, const cg_field* C, const cg_field* q, double dt,
                                 const cg_mask* m) {
    if (C->dtype == CG_F64) diffusion_update_C_masked_t<double>(grid, C, q, dt, m);
    else diffusion_update_C_masked_t<float>(grid, C, q, dt, m);
    return CG_OK;
}

int or_diffusion_update_C(const cg_grid* grid, const cg_field* C, const cg_field* q, double dt) {
    if (C->dtype == CG_F64) diffusion_update_C_t<double>(grid, C, q, dt);
    else diffusion_update_C_t<float>(grid, C, q, dt);
    return CG_OK;
}

int or_stokes_update_old(const cg_grid* grid, const cg_stokes_fields* f) {
    if (f->tau[0].dtype == CG_F64) stokes_update_old_t<double>(grid, f);
    else stokes_update_old_t<float>(grid, f);
    return CG_OK;
}

int or_stokes_update_stress(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p) {
    if (f->tau[0].dtype == CG_F64) stokes_update_stress_t<double>(grid, f, p);
    else stokes_update_stress_t<float>(grid, f, p);
    return CG_OK;
}

int or_stokes_update_velocity(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p) {
    if (f->tau[0].dtype == CG_F64) stokes_update_velocity_t<double>(grid, f, p);
    else stokes_update_velocity_t<float>(grid, f, p);
    return CG_OK;
}

/* The Stokes kernels with the masked operators (every derivative's operands weighted by the
 * FieldMask at their location and index). */
int or_stokes_update_stress_masked(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
                                   const cg_mask* mask) {
    if (f->tau[0].dtype == CG_F64) stokes_update_stress_t<double>(grid, f, p, mask);
    else stokes_update_stress_t<float>(grid, f, p, mask);
    return 0;
}

int or_stokes_update_velocity_masked(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p,
                                     const cg_mask* mask) {
    if (f->tau[0].dtype == CG_F64) stokes_update_velocity_t<double>(grid, f, p, mask);
    else stokes_update_velocity_t<float>(grid, f, p, mask);
    return 0;
}

int or_stokes_update_thermal_flux(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p) {
    if (!f->T.data || !f->qT[0].data || !f->qT[1].data || (grid->ndim > 2 && !f->qT[2].data)) return CG_ERR_ARG;
    if (f->T.dtype == CG_F64) stokes_update_thermal_flux_t<double>(grid, f, p);
    else stokes_update_thermal_flux_t<float>(grid, f, p);
    return CG_OK;
}

int or_stokes_update_thermal(const cg_grid* grid, const cg_stokes_fields* f, const cg_stokes_params* p) {
    if (!f->T.data || !f->T_old.data || !f->qT[0].data || !f->qT[1].data || (grid->ndim > 2 && !f->qT[2].data))
        return CG_ERR_ARG;
    if (f->T.dtype == CG_F64) stokes_update_thermal_t<double>(grid, f, p);
    else stokes_update_thermal_t<float>(grid, f, p);
    return CG_OK;
}

int or_ptdiff_update_q(const cg_grid* grid, const cg_ptdiff_fields* f, const cg_ptdiff_params* p) {
    if (f->C.dtype == CG_F64) ptdiff_update_q_t<double>(grid, f, p);
    else ptdiff_update_q_t<float>(grid, f, p);
    return CG_OK;
}

int or_ptdiff_update_C(const cg_grid* grid, const cg_ptdiff_fields* f, const cg_ptdiff_params* p) {
    if (f->C.dtype == CG_F64) ptdiff_update_C_t<double>(grid, f, p);
    else ptdiff_update_C_t<float>(grid, f, p);
    return CG_OK;
}

int or_sia_update_q(const cg_grid* grid, const cg_field* q, const cg_field* H, const cg_field* B,
                    const cg_sia_params* p, double* dmax) {
    if (H->dtype == CG_F64) sia_update_q_t<double>(grid, q, H, B, p, dmax);
    else sia_update_q_t<float>(grid, q, H, B, p, dmax);
    return CG_OK;
}

int or_sia_update_H(const cg_grid* grid, const cg_field* H, const cg_field* q, const cg_field* B, double dt,
                    const cg_sia_params* p) {
    if (H->dtype == CG_F64) sia_update_H_t<double>(grid, H, q, B, dt, p);
    else sia_update_H_t<float>(grid, H, q, B, dt, p);
    return CG_OK;
}

int or_op_kernel(int op, const cg_grid* grid, const cg_field* C, const cg_field* C1, const cg_field* C2,
                 const cg_field* V, const cg_field* chi) {
    const cg_field* any = C ? C : (C1 ? C1 : V);
    if (any->dtype == CG_F64) op_kernel_t<double>(op, grid, C, C1, C2, V, chi);
    else op_kernel_t<float>(op, grid, C, C1, C2, V, chi);
    return CG_OK;
}

}  // extern "C"
