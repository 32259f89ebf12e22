// Fused Runge-Kutta stage kernel and the small per-step kernels.
//
// One launch of stage_kernel advances one RK stage of the whole grid: each CTA
// stages its tile plus a halo of g cells of every conserved variable in shared
// memory, reconstructs each direction, evaluates the face fluxes, forms the
// flux difference L (the reference's computeFlux output: sum over directions
// of F_{i-1/2} - F_{i+1/2}, unscaled), combines it with the stage inputs as the
// reference integrators do, and writes the cell together with its ghost
// images (the Neumann / periodic boundary as an index map), so the next stage
// reads a complete padded array. Face wave speeds are reduced by warp shuffles
// and one atomic per CTA and direction.
//
// Stage modes (RK3 = SSP-RK3, RK2 = SSP-RK2, FE = forward Euler, c = dt/dx.x):
//   MODE_L        in = U                 out = L(in)           (stage 0 of all)
//   MODE_RK3_S1   in = L0*c + U0         out = ((L(in)*c + in)*(1/3) + U0)*(3/4)
//   MODE_RK3_S2   in = U                 out = ((L(in)*c + in)*2 + U0)*(1/3)
//   MODE_RK2_S1   in = L0*c + U0         out = ((L(in)*c + in) + U0)*0.5
// (alsfvm/src/integrator/RungeKutta3.cpp:49-86, RungeKutta2.cpp:37-67). Stage 1
// rebuilds U1 on the fly from U0 and L0, so U1 is never stored and an RK3 step
// moves the algorithmic 8 * nvar state words per cell.
#pragma once
#include <type_traits>

#include "fv_df.cuh"
#include "fv_math.cuh"
#include "fv_tma.cuh"
#include "fv_types.h"

namespace gbfv {
namespace GBFV_VARIANT_NS {

template <class R> __device__ __forceinline__ R mul_rn(R a, R b);
template <> __device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <class R> __device__ __forceinline__ R add_rn(R a, R b);
template <> __device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }

// a * b + c: two IEEE roundings in the exact policy (the reference's
// `out *= c; out += u`), one fused rounding otherwise
template <class R> __device__ __forceinline__ R madd(R a, R b, R c) {
    if constexpr (kExact)
        return add_rn(mul_rn(a, b), c);
    else
        return fma(a, b, c);
}

template <class C> __device__ __forceinline__ C shfl_xor_c(C v, int off) {
    return __shfl_xor_sync(0xffffffffu, v, off);
}
template <> __device__ __forceinline__ dfloat shfl_xor_c<dfloat>(dfloat v, int off) {
    return dfloat(__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off));
}

// A kernel-uniform double in the arithmetic type: the float copy the host or
// the dt kernel rounded once (no per-thread conversion on the FP64 pipe), the
// double itself, or its double-float split.
template <class T> __device__ __forceinline__ T uniform_value(double d, float f);
template <> __device__ __forceinline__ double uniform_value<double>(double d, float) { return d; }
template <> __device__ __forceinline__ float uniform_value<float>(double, float f) { return f; }
template <> __device__ __forceinline__ dfloat uniform_value<dfloat>(double d, float) { return dfloat(d); }

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
    atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// Conserved-variable count and the flux between two reconstructed states.
template <class R, int EQ, int FLUX> struct Physics {
    static constexpr int NSD = EQ == 0 ? 1 : EQ;
    static constexpr int NV = EQ == 0 ? 1 : EQ + 2;
    template <int D>
    static __device__ __forceinline__ R face_flux(const R* a, const R* b, R gamma, R* F) {
        if constexpr (EQ == 0) {
            if constexpr (FLUX == 2)
                return flux_godunov<R>(a[0], b[0], F);
            else
                return flux_burgers<R, FLUX>(a[0], b[0], F);
        } else {
            EulerState<R, NSD> L, Rr;
            L.rho = a[0];
            Rr.rho = b[0];
#pragma unroll
            for (int k = 0; k < NSD; ++k) {
                L.m[k] = a[1 + k];
                Rr.m[k] = b[1 + k];
            }
            L.E = a[1 + NSD];
            Rr.E = b[1 + NSD];
            euler_extra<R, NSD>(L, gamma);
            euler_extra<R, NSD>(Rr, gamma);
            if constexpr (FLUX == 1)
                return flux_hll3<R, NSD, D>(L, Rr, gamma, F);
            else if constexpr (FLUX == 3)
                return flux_central<R, NSD, D>(L, Rr, gamma, F);
            else
                return flux_hll<R, NSD, D>(L, Rr, gamma, F);
        }
    }
    // Constraint check of one cell (CPUCellComputer::obeysConstraints,
    // alsfvm/src/equation/CPUCellComputer.cpp:79-125): finite values, rho > 0, p > 0.
    static __device__ __forceinline__ bool obeys(const R* c, R gamma) {
        if constexpr (EQ == 0) {
            return isfinite(c[0]);
        } else {
            EulerState<R, NSD> s;
            s.rho = c[0];
#pragma unroll
            for (int k = 0; k < NSD; ++k) s.m[k] = c[1 + k];
            s.E = c[1 + NSD];
            euler_extra<R, NSD>(s, gamma);
            bool ok = isfinite(s.rho) && isfinite(s.E) && isfinite(s.p) && gt0(s.rho) && gt0(s.p);
#pragma unroll
            for (int k = 0; k < NSD; ++k) ok = ok && isfinite(s.m[k]) && isfinite(s.u[k]);
            return ok;
        }
    }
};

template <int DIM, int TX, int TY, int TZ> struct Tile {
    static constexpr int NT = TX * TY * TZ;
    static constexpr int T[3] = {TX, TY, TZ};
};

// Line buffers keep each item's values together so that a reconstruction's,
// a face's or a cell's values move with 128-bit shared-memory accesses: one
// to four per item instead of NV scalar accesses. The first VEC values of an
// item sit item-major in 16-byte vectors; when NV leaves a remainder of more
// than one value short of a whole vector (five floats: 4 + 1), the remainder
// (TAIL values per item) sits item-major in a second array after the first,
// so no item carries more than one value of padding. A buffer holds CAP
// items (the capacity rounded up to a multiple of 4, which keeps both parts
// and the next buffer 16-byte aligned).
template <class R, int NV> struct LinePad {
    static constexpr int per16 = (int)(16 / sizeof(R));
    static constexpr int rem = NV % per16;
    static constexpr bool split = NV > 1 && rem != 0 && per16 - rem > 1;
    static constexpr int VEC = NV == 1 ? 1 : (split ? NV - rem : ((NV + per16 - 1) / per16) * per16);
    static constexpr int TAIL = split ? rem : 0;
    static constexpr int value = VEC + TAIL;  // values per item
    static constexpr int cap(int items) { return (items + 3) / 4 * 4; }
};

template <int NV, class R> __device__ __forceinline__ R lane_or_zero(const R* v, int i) {
    return i < NV ? v[i < NV ? i : 0] : R(0);
}

// Item `item` of a line buffer of CAP items at `base` (16-byte aligned).
template <class R, int NV, int CAP> __device__ __forceinline__ void line_put(R* base, int item, const R* v) {
    using LP = LinePad<R, NV>;
    constexpr int P = LP::VEC;
    R* p = base + item * P;
    if constexpr (NV == 1) {
        p[0] = v[0];
    } else if constexpr (std::is_same<R, float>::value) {
#pragma unroll
        for (int c = 0; c < P / 4; ++c)
            reinterpret_cast<float4*>(p)[c] =
                make_float4(lane_or_zero<NV>(v, 4 * c), lane_or_zero<NV>(v, 4 * c + 1),
                            lane_or_zero<NV>(v, 4 * c + 2), lane_or_zero<NV>(v, 4 * c + 3));
    } else if constexpr (std::is_same<R, double>::value) {
#pragma unroll
        for (int c = 0; c < P / 2; ++c)
            reinterpret_cast<double2*>(p)[c] = make_double2(lane_or_zero<NV>(v, 2 * c), lane_or_zero<NV>(v, 2 * c + 1));
    } else {  // double-float: two pairs per 16 bytes
#pragma unroll
        for (int c = 0; c < P / 2; ++c) {
            const R a = lane_or_zero<NV>(v, 2 * c), b = lane_or_zero<NV>(v, 2 * c + 1);
            reinterpret_cast<float4*>(p)[c] = make_float4(a.hi, a.lo, b.hi, b.lo);
        }
    }
    if constexpr (LP::TAIL > 0) {
        R* t = base + CAP * P + item * LP::TAIL;
#pragma unroll
        for (int k = 0; k < LP::TAIL; ++k) t[k] = v[P + k];
    }
}

template <class R, int NV, int CAP> __device__ __forceinline__ void line_get(const R* base, int item, R* v) {
    using LP = LinePad<R, NV>;
    constexpr int P = LP::VEC;
    const R* p = base + item * P;
    if constexpr (NV == 1) {
        v[0] = p[0];
    } else if constexpr (std::is_same<R, float>::value) {
#pragma unroll
        for (int c = 0; c < P / 4; ++c) {
            const float4 q = reinterpret_cast<const float4*>(p)[c];
            if (4 * c < NV) v[4 * c < NV ? 4 * c : 0] = q.x;
            if (4 * c + 1 < NV) v[4 * c + 1 < NV ? 4 * c + 1 : 0] = q.y;
            if (4 * c + 2 < NV) v[4 * c + 2 < NV ? 4 * c + 2 : 0] = q.z;
            if (4 * c + 3 < NV) v[4 * c + 3 < NV ? 4 * c + 3 : 0] = q.w;
        }
    } else if constexpr (std::is_same<R, double>::value) {
#pragma unroll
        for (int c = 0; c < P / 2; ++c) {
            const double2 q = reinterpret_cast<const double2*>(p)[c];
            if (2 * c < NV) v[2 * c < NV ? 2 * c : 0] = q.x;
            if (2 * c + 1 < NV) v[2 * c + 1 < NV ? 2 * c + 1 : 0] = q.y;
        }
    } else {
#pragma unroll
        for (int c = 0; c < P / 2; ++c) {
            const float4 q = reinterpret_cast<const float4*>(p)[c];
            if (2 * c < NV) v[2 * c < NV ? 2 * c : 0] = R(q.x, q.y);
            if (2 * c + 1 < NV) v[2 * c + 1 < NV ? 2 * c + 1 : 0] = R(q.z, q.w);
        }
    }
    if constexpr (LP::TAIL > 0) {
        const R* t = base + CAP * P + item * LP::TAIL;
#pragma unroll
        for (int k = 0; k < LP::TAIL; ++k) v[P + k] = t[k];
    }
}

template <class R, int NV, int G, int DIM, int TX, int TY, int TZ>
struct SmemLayout {
    static constexpr int GX = G, GY = DIM > 1 ? G : 0, GZ = DIM > 2 ? G : 0;
    static constexpr int HX = TX + 2 * GX, HY = TY + 2 * GY, HZ = TZ + 2 * GZ;
    static constexpr int HALO = HX * HY * HZ;
    // per-direction line buffers: reconstructed left/right values of the
    // (T_d + 2) cells along d, times the tile's extent in the other
    // dimensions; each face flux overwrites the right value it consumed
    static constexpr int REC0 = (TX + 2) * TY * TZ;
    static constexpr int REC1 = DIM > 1 ? TX * (TY + 2) * TZ : 0;
    static constexpr int REC2 = DIM > 2 ? TX * TY * (TZ + 2) : 0;
    static constexpr int REC = REC0 > REC1 ? (REC0 > REC2 ? REC0 : REC2) : (REC1 > REC2 ? REC1 : REC2);
    static constexpr size_t round128(size_t b) { return (b + 127) & ~(size_t)127; }
    static constexpr size_t box_bytes = sizeof(R) * (size_t)NV * HALO;  // one halo of every variable
    static constexpr size_t halo_bytes = round128(box_bytes);           // its slot (TMA wants 128 B aligned)
    static constexpr int CAP = LinePad<R, NV>::cap(REC);  // items per line buffer
    static constexpr int LINE = LinePad<R, NV>::value * CAP;  // values per line buffer
    static constexpr size_t work_bytes = sizeof(R) * (2 * (size_t)LINE);
    // Dynamic shared memory per kernel, plus 128 bytes to align the base:
    //   plain staging:    halo | line buffers
    //   TMA staging:      halo | line buffers, which first hold the L0 halo of the stage-1 modes
    //   ensemble (R = C): halo A | halo B | L0 halo | line buffers
    static constexpr size_t bytes = 128 + halo_bytes + work_bytes;
    static constexpr size_t tma_bytes = 128 + halo_bytes + (work_bytes > halo_bytes ? work_bytes : halo_bytes);
    static constexpr size_t pipe_bytes = 128 + 3 * halo_bytes + work_bytes;
};

// The dynamic shared memory base rounded up to 128 bytes.
__device__ __forceinline__ unsigned char* align_smem(unsigned char* p) {
    return p + ((128u - (smem_addr(p) & 127u)) & 127u);
}

// Cells of the tile each thread owns in the accumulate and combine phases:
// thread t owns cells t, t + NTH, ... (NTH >= cells: one cell for the first
// `cells` threads; the rest join the reconstruction and flux phases only).
template <int NT, int NTH> struct CellsPerThread {
    static_assert(NTH % 32 == 0, "whole warps");
    static_assert(NT <= NTH || NT % NTH == 0, "a whole number of cells per thread");
    static constexpr int value = NT <= NTH ? 1 : NT / NTH;
};


// One direction D of the tile: reconstruct, face fluxes, accumulate into acc.
// A face counts towards the wave-speed maximum when its cells along D lie
// in [0, hi[D]] (faces 0 .. n of the grid, or of a region's cells) and the
// other coordinates below hi.
template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH, int D>
__device__ __forceinline__ void tile_direction(const R* su, R* rl, R* rr, R* acc, int tid,
                                               const int* org, const int* hi, R gamma, R& wsmax) {
    using Ph = Physics<R, EQ, FLUX>;
    constexpr int NV = Ph::NV;
    using SL = SmemLayout<R, NV, ReconTraits<RC>::ghosts, DIM, TX, TY, TZ>;
    constexpr int NT = TX * TY * TZ;  // cells of the tile
    constexpr int TD = D == 0 ? TX : (D == 1 ? TY : TZ);
    constexpr int O1 = D == 0 ? TY : TX;          // extent of the first other dimension
    constexpr int LEN = TD + 2;
    constexpr int NREC = LEN * (NT / TD);
    constexpr int NFACE = (TD + 1) * (NT / TD);
    constexpr int DS = D == 0 ? 1 : (D == 1 ? SL::HX : SL::HX * SL::HY);
    constexpr int VS = SL::HALO;
    constexpr int CAP = SL::CAP;
    (void)NREC;

    // Work items: along x (D = 0) the cells of a line are consecutive; for
    // D >= 1 consecutive items step along x (p, the first other dimension),
    // so a warp's shared-memory accesses stay unit-stride in every phase.
    // Line buffers hold item w at slot w in both layouts:
    //   D = 0:  w = (o * LEN + a),            o = p + O1 q
    //   D >= 1: w = ((q * LEN + a) * O1 + p)  (faces: LEN -> TD + 1)
    // reconstruction of cells -1 .. TD along D
    for (int w = tid; w < NREC; w += NTH) {
        int a, p, q;
        if constexpr (D == 0) {
            a = w % LEN;
            const int o = w / LEN;
            p = o % O1;
            q = o / O1;
        } else {
            p = w % O1;
            const int r = w / O1;
            a = r % LEN;
            q = r / LEN;
        }
        int c[3];
        c[D] = a - 1;
        if (D == 0) { c[1] = p; c[2] = q; }
        else if (D == 1) { c[0] = p; c[2] = q; }
        else { c[0] = p; c[1] = q; }
        const int s = ((c[2] + SL::GZ) * SL::HY + (c[1] + SL::GY)) * SL::HX + (c[0] + SL::GX);
        R l[NV], r[NV];
        reconstruct_cell<R, NV, RC>(su + s, VS, DS, l, r, gamma);
        line_put<R, NV, CAP>(rl, w, l);
        line_put<R, NV, CAP>(rr, w, r);
    }
    __syncthreads();
    // face b is the left face of tile cell b along D (between cells b-1 and b)
    for (int f = tid; f < NFACE; f += NTH) {
        int b, p, q, il, ir;  // il: item of cell b-1, ir: item of cell b
        if constexpr (D == 0) {
            b = f % (TD + 1);
            const int o = f / (TD + 1);
            p = o % O1;
            q = o / O1;
            il = o * LEN + b;
            ir = il + 1;
        } else {
            p = f % O1;
            const int r = f / O1;
            b = r % (TD + 1);
            q = r / (TD + 1);
            il = (q * LEN + b) * O1 + p;
            ir = il + O1;
        }
        R a[NV], bb[NV], F[NV];
        line_get<R, NV, CAP>(rr, il, a);   // cell b-1 at its right face
        line_get<R, NV, CAP>(rl, ir, bb);  // cell b at its left face
        const R w = Ph::template face_flux<D>(a, bb, gamma, F);
        // the flux of face b replaces the right value of cell b - 1 (item il),
        // which no other face reads
        line_put<R, NV, CAP>(rr, il, F);
        // the face counts if both neighbours lie in the grid's interior range
        int c[3];
        c[D] = b;
        if (D == 0) { c[1] = p; c[2] = q; }
        else if (D == 1) { c[0] = p; c[2] = q; }
        else { c[0] = p; c[1] = q; }
        bool valid = org[D] + c[D] <= hi[D];
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (d != D) valid = valid && (org[d] + c[d] < hi[d]);
        if (valid) wsmax = fmax_(wsmax, w);
    }
    __syncthreads();
    // this thread's cells: acc += (-F_{i+1/2}) + F_{i-1/2}
    constexpr int CPT = CellsPerThread<NT, NTH>::value;
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
        const int cell = tid + j * NTH;
        if (cell >= NT) continue;
        const int cx = cell % TX, cy = (cell / TX) % TY, cz = cell / (TX * TY);
        const int cd = D == 0 ? cx : (D == 1 ? cy : cz);
        const int p = D == 0 ? cy : cx;
        const int q = D == 2 ? cy : cz;
        // faces cd (left) and cd + 1 (right) of this cell's line, stored at
        // the items of cells cd - 1 and cd
        const int fli = D == 0 ? (p + O1 * q) * LEN + cd : (q * LEN + cd) * O1 + p;
        const int fri = D == 0 ? fli + 1 : fli + O1;
        R FL[NV], FR[NV];
        line_get<R, NV, CAP>(rr, fli, FL);
        line_get<R, NV, CAP>(rr, fri, FR);
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const R fl = FL[k];
            const R fr = FR[k];
            if constexpr (!kExact && D == 0)
                acc[j * NV + k] = fl - fr;  // the first direction starts the sum
            else
                acc[j * NV + k] = acc[j * NV + k] + ((-fr) + fl);
        }
    }
    __syncthreads();
}

// One tile of one stage: shared by the single-grid kernel (one CTA per tile)
// and the persistent ensemble kernel (each CTA loops over a list of tiles of
// many grids). Every thread of the CTA calls it; it synchronises internally.
// R is the storage type of the state in HBM, C the type the reconstruction and
// flux arithmetic runs in (C = R, or the double-float type for an FP64 state).
// With C != R the combination with the stage inputs re-reads the exact R
// values of the thread's own cell (L1/L2 hits: the tile load just fetched them)
// and runs in R.
// Phase 1 of a tile: the tile plus its halo of g cells per active dimension
// into su, the stage-1 modes forming U1 = L0 c + U0 on the way.
// REGION: the region kernel's load, one input array per variable (A.vin).
template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH, class C = R, bool REGION = false>
__device__ __forceinline__ void stage_tile_load(const StageArgs& A, const int* org, C* su) {
    constexpr int NV = Physics<C, EQ, FLUX>::NV;
    using SL = SmemLayout<C, NV, ReconTraits<RC>::ghosts, DIM, TX, TY, TZ>;
    constexpr bool kSame = std::is_same<R, C>::value;
    const Grid& Gd = A.G;
    const int tid = threadIdx.x;
    const R* in = reinterpret_cast<const R*>(A.in);
    const R* l0 = reinterpret_cast<const R*>(A.l0);
    const long long total = Gd.total;
    const int mode = A.mode;
    const R scale = uniform_value<R>(A.st->scale, A.st->scale_f);
    for (int w = tid; w < SL::HALO; w += NTH) {
        const int hx = w % SL::HX, hy = (w / SL::HX) % SL::HY, hz = w / (SL::HX * SL::HY);
        const int px = org[0] + hx, py = org[1] + hy, pz = org[2] + hz;
        if (px < Gd.t[0] && py < Gd.t[1] && pz < Gd.t[2]) {
            const long long gi = gidx(Gd, px, py, pz);
            if constexpr (REGION) {
#pragma unroll
                for (int k = 0; k < NV; ++k) su[k * SL::HALO + w] = C(reinterpret_cast<const R*>(A.vin[k])[gi]);
            } else {
#pragma unroll
                for (int k = 0; k < NV; ++k) {
                    // U1 = L0 * c + U0 (the reference's *= then +=), formed in R:
                    // the ENO stencil choices compare differences of these values
                    const R v = (mode == MODE_RK3_S1 || mode == MODE_RK2_S1)
                                    ? madd(l0[k * total + gi], scale, in[k * total + gi])
                                    : in[k * total + gi];
                    su[k * SL::HALO + w] = C(v);
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) su[k * SL::HALO + w] = C(1);
        }
    }
    (void)kSame;
    __syncthreads();
}

// Asynchronous copy of one element global -> shared (cp.async, sm_80+): the
// ensemble kernel stages the next tile's halo while the current one computes.
template <class T> __device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Issues the copies of a tile's halo into su (and of L0 into l0s for the
// stage-1 modes); cells past the padded array get the values the
// synchronous load gives them. Storage and arithmetic type must agree.
template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH>
__device__ __forceinline__ void stage_tile_prefetch(const StageArgs& A, const int* org, R* su, R* l0s) {
    constexpr int NV = Physics<R, EQ, FLUX>::NV;
    using SL = SmemLayout<R, NV, ReconTraits<RC>::ghosts, DIM, TX, TY, TZ>;
    const Grid& Gd = A.G;
    const int tid = threadIdx.x;
    const R* in = reinterpret_cast<const R*>(A.in);
    const R* l0 = reinterpret_cast<const R*>(A.l0);
    const long long total = Gd.total;
    const bool s1 = A.mode == MODE_RK3_S1 || A.mode == MODE_RK2_S1;
    for (int w = tid; w < SL::HALO; w += NTH) {
        const int hx = w % SL::HX, hy = (w / SL::HX) % SL::HY, hz = w / (SL::HX * SL::HY);
        const int px = org[0] + hx, py = org[1] + hy, pz = org[2] + hz;
        if (px < Gd.t[0] && py < Gd.t[1] && pz < Gd.t[2]) {
            const long long gi = gidx(Gd, px, py, pz);
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                cp_async_elem(su + k * SL::HALO + w, in + k * total + gi);
                if (s1) cp_async_elem(l0s + k * SL::HALO + w, l0 + k * total + gi);
            }
        } else {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                su[k * SL::HALO + w] = R(1);
                if (s1) l0s[k * SL::HALO + w] = R(0);  // L0 c + 1 = 1
            }
        }
    }
    cp_async_commit();
}

// Waits for the prefetched halo; the stage-1 modes then form U1 = L0 c + U0.
template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH>
__device__ __forceinline__ void stage_tile_prefetch_finish(const StageArgs& A, R* su, const R* l0s) {
    constexpr int NV = Physics<R, EQ, FLUX>::NV;
    using SL = SmemLayout<R, NV, ReconTraits<RC>::ghosts, DIM, TX, TY, TZ>;
    cp_async_wait_all();
    __syncthreads();
    if (A.mode == MODE_RK3_S1 || A.mode == MODE_RK2_S1) {
        const R scale = uniform_value<R>(A.st->scale, A.st->scale_f);
        for (int w = threadIdx.x; w < SL::HALO; w += NTH) {
#pragma unroll
            for (int k = 0; k < NV; ++k) su[k * SL::HALO + w] = madd(l0s[k * SL::HALO + w], scale, su[k * SL::HALO + w]);
        }
        __syncthreads();
    }
}

// Phases 2-4 of a tile whose halo is in su; work holds the per-direction
// line buffers (reconstructed face values and face fluxes).
// REGION: the region kernel (MODE_L over the cells [A.rlo, A.rhi), faces
// and stores limited to them, one output array per variable, no ghost
// images written).
template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH, class C = R, bool REGION = false>
__device__ __forceinline__ void stage_tile_compute(const StageArgs& A, const int* org, const C* su, C* work,
                                                   C* wred) {
    using Ph = Physics<C, EQ, FLUX>;
    using PhR = Physics<R, EQ, FLUX>;
    constexpr int NV = Ph::NV;
    constexpr int G = ReconTraits<RC>::ghosts;
    using SL = SmemLayout<C, NV, G, DIM, TX, TY, TZ>;
    constexpr int NT = TX * TY * TZ;  // cells of the tile
    constexpr int CPT = CellsPerThread<NT, NTH>::value;
    constexpr bool kSame = std::is_same<R, C>::value;
    C* rl = work;
    C* rr = rl + SL::LINE;

    const Grid& Gd = A.G;
    const int tid = threadIdx.x;
    const R* in = reinterpret_cast<const R*>(A.in);
    const R* u0 = reinterpret_cast<const R*>(A.u0);
    const R* l0 = reinterpret_cast<const R*>(A.l0);
    R* out = reinterpret_cast<R*>(A.out);
    const long long total = Gd.total;
    const int mode = A.mode;
    const R scale = uniform_value<R>(A.st->scale, A.st->scale_f);
    const int* hi = REGION ? A.rhi : Gd.n;  // cells and faces at or past hi are not this launch's

    // The combination at the end reads U0 of the thread's cells from global
    // memory (and, with per-thread staging of another type, the stage input):
    // start those lines towards L1 now so they arrive during the compute.
    if (mode != MODE_L) {
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
            const int cell = tid + j * NTH;
            if (cell >= NT) continue;
            const int ix = org[0] + cell % TX, iy = org[1] + (cell / TX) % TY, iz = org[2] + cell / (TX * TY);
            if (ix >= Gd.n[0] || iy >= Gd.n[1] || iz >= Gd.n[2]) continue;
            const long long own = gidx(Gd, ix + Gd.g[0], iy + Gd.g[1], iz + Gd.g[2]);
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                asm volatile("prefetch.global.L1 [%0];\n" ::"l"(u0 + k * total + own));
                if constexpr (!kSame) asm volatile("prefetch.global.L1 [%0];\n" ::"l"(in + k * total + own));
            }
        }
    }

    // 2. flux difference per direction, per owned cell
    C acc[CPT * NV];
#pragma unroll
    for (int k = 0; k < CPT * NV; ++k) acc[k] = C(0);
    // wave-speed maxima in the arithmetic type (the max is exact, so one
    // conversion per thread gives the same double as converting every face)
    C wsd[3] = {C(0), C(0), C(0)};
    const C gamma = uniform_value<C>(A.gamma, A.gamma_f);
    tile_direction<C, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, 0>(su, rl, rr, acc, tid, org, hi, gamma, wsd[0]);
    if constexpr (DIM > 1)
        tile_direction<C, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, 1>(su, rl, rr, acc, tid, org, hi, gamma, wsd[1]);
    if constexpr (DIM > 2)
        tile_direction<C, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, 2>(su, rl, rr, acc, tid, org, hi, gamma, wsd[2]);

    // 3. wave speeds (stage 0 only): warp max, CTA max, one atomic per direction
    if (mode == MODE_L) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            C v = wsd[d];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v = fmax_(v, shfl_xor_c(v, off));
            if ((tid & 31) == 0) wred[(tid >> 5) * 3 + d] = v;
        }
        __syncthreads();
        // one conversion to double per CTA and direction: per-warp FP64
        // instructions occupy GB300's narrow FP64 pipe even on one lane
        if (tid < DIM) {
            C v = wred[tid];
            for (int w = 1; w < NTH / 32; ++w) v = fmax_(v, wred[w * 3 + tid]);
            atomic_max_nonneg(&A.st->ws_bits[tid], (double)v);
        }
    }

    // 4. this thread's cells: combine and write with their ghost images (no
    // barrier follows)
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
    const int cell = tid + j * NTH;
    if (cell >= NT) continue;
    const int cx = cell % TX, cy = (cell / TX) % TY, cz = cell / (TX * TY);
    const int ix = org[0] + cx, iy = org[1] + cy, iz = org[2] + cz;
    if (ix >= hi[0] || iy >= hi[1] || iz >= hi[2]) continue;
    const int sidx = ((cz + SL::GZ) * SL::HY + (cy + SL::GY)) * SL::HX + (cx + SL::GX);
    const long long own = gidx(Gd, ix + Gd.g[0], iy + Gd.g[1], iz + Gd.g[2]);
    if constexpr (REGION) {
#pragma unroll
        for (int k = 0; k < NV; ++k) reinterpret_cast<R*>(A.vout[k])[own] = (R)acc[j * NV + k];
    } else {
    R res[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const R acck = (R)acc[j * NV + k];
        if (mode == MODE_L) {
            res[k] = acck;
        } else {
            R uin;
            if constexpr (kSame) {
                uin = su[k * SL::HALO + sidx];
            } else if (mode == MODE_RK3_S1 || mode == MODE_RK2_S1) {
                uin = madd(l0[k * total + own], scale, in[k * total + own]);
            } else {
                uin = in[k * total + own];
            }
            const R base = u0[k * total + own];
            R v = madd(acck, scale, uin);
            if (mode == MODE_RK3_S1) {
                v = madd(v, R(1. / 3.), base);
                v = mul_rn(v, R(3. / 4.));
            } else if (mode == MODE_RK3_S2) {
                v = madd(v, R(2), base);
                v = mul_rn(v, R(1. / 3.));
            } else {  // MODE_RK2_S1
                v = add_rn(v, base);
                v = mul_rn(v, R(0.5));
            }
            res[k] = v;
        }
    }
    if (A.check && !PhR::obeys(res, uniform_value<R>(A.gamma, A.gamma_f))) {
        if (atomicCAS(&A.st->status, 0, 1) == 0) A.st->failed_step = (int)A.st->steps + 1;
    }
    store_with_images<R, NV>(out, total, Gd, ix, iy, iz, A.periodic != 0, res);
    if (A.out2) store_with_images<R, NV>(reinterpret_cast<R*>(A.out2), total, Gd, ix, iy, iz, A.periodic != 0, res);
    if constexpr (kSame) {
        if (A.copy_in) {
            R vin[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) vin[k] = su[k * SL::HALO + sidx];
            store_with_images<R, NV>(reinterpret_cast<R*>(A.copy_in), total, Gd, ix, iy, iz, A.periodic != 0, vin);
        }
    }
    }
    }
}

// TMA staging of one tile (thread 0 only): the halo box of the stage input
// into su and, for the stage-1 modes, that of L0 into l0s, both signalling
// bar. `global_maps`: the maps live in global memory, written by the host.
template <class R, class SL, int DIM>
// `extra_tx`: bytes announced on top of the copies' (0; a test of the bounded
// wait's error path announces more than arrives, so the wait runs out).
__device__ __forceinline__ void tma_stage_issue(const StageArgs& A, const CUtensorMap* tm_in, const CUtensorMap* tm_l0,
                                                const int* org, R* su, R* l0s, unsigned long long* bar,
                                                bool global_maps, unsigned extra_tx = 0) {
    const bool s1 = A.mode == MODE_RK3_S1 || A.mode == MODE_RK2_S1;
    if (global_maps) {
        fence_tensormap_acquire(tm_in);
        if (s1) fence_tensormap_acquire(tm_l0);
    }
    // earlier generic accesses of su / l0s (the previous tile) before the copies
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, (unsigned)((s1 ? 2 : 1) * SL::box_bytes) + extra_tx);
    tma_load_halo<DIM>(su, tm_in, bar, org[0], org[1], org[2]);
    if (s1) tma_load_halo<DIM>(l0s, tm_l0, bar, org[0], org[1], org[2]);
}

// Every thread: waits for the TMA staging of phase `phase`, then the stage-1
// modes form U1 = L0 c + U0 in su. Returns false (the same for every thread)
// when the copies did not complete within the time limit; the step state then
// records kStatusTmaTimeout and the caller returns without touching su.
template <class R, class SL, int NTH>
__device__ __forceinline__ bool tma_stage_finish(const StageArgs& A, R* su, const R* l0s, unsigned long long* bar,
                                                 unsigned phase) {
    constexpr int NV = (int)(SL::box_bytes / (sizeof(R) * SL::HALO));
    if (!__syncthreads_and(mbar_wait_bounded(bar, phase))) {
        if (threadIdx.x == 0 && atomicCAS(&A.st->status, 0, kStatusTmaTimeout) == 0)
            A.st->failed_step = (int)A.st->steps + 1;
        mbar_wait_bounded(bar, phase);  // copies still in flight get the time limit once more
        return false;
    }
    if (A.mode == MODE_RK3_S1 || A.mode == MODE_RK2_S1) {
        const R scale = uniform_value<R>(A.st->scale, A.st->scale_f);
        for (int w = threadIdx.x; w < SL::HALO; w += NTH) {
#pragma unroll
            for (int k = 0; k < NV; ++k) su[k * SL::HALO + w] = madd(l0s[k * SL::HALO + w], scale, su[k * SL::HALO + w]);
        }
        __syncthreads();
    }
    return true;
}

// One tile of one stage with a synchronous halo load. Shared memory: the halo
// tile, then the line buffers.
template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH, class C = R>
__device__ __forceinline__ void stage_tile(const StageArgs& A, const int* org, unsigned char* base, C* wred) {
    constexpr int NV = Physics<C, EQ, FLUX>::NV;
    using SL = SmemLayout<C, NV, ReconTraits<RC>::ghosts, DIM, TX, TY, TZ>;
    C* su = reinterpret_cast<C*>(base);
    stage_tile_load<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, C>(A, org, su);
    stage_tile_compute<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, C>(A, org, su,
                                                                 reinterpret_cast<C*>(base + SL::halo_bytes), wred);
}

template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH, class C = R, int MINB = 1>
__global__ void __launch_bounds__(NTH, MINB) stage_kernel(StageArgs A) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned char wred_raw[(NTH / 32) * 3 * sizeof(C)];
    C* wred = reinterpret_cast<C*>(wred_raw);
    if (A.st->done) return;
    const int org[3] = {(int)blockIdx.x * TX, (int)blockIdx.y * TY, (int)blockIdx.z * TZ};
    stage_tile<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, C>(A, org, align_smem(smem_raw), wred);
}

// The operator on a region of the grid (NumericalFlux::computeFlux with start
// / end, alsfvm/src/numflux/NumericalFluxCPU.cpp:167-221): the default tile
// with per-thread loads, tiles starting at the region's first cell, MODE_L
// into A.vout; the wave speeds of the region's faces into A.st.
template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH, class C = R>
__global__ void __launch_bounds__(NTH, 1) region_kernel(StageArgs A) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned char wred_raw[(NTH / 32) * 3 * sizeof(C)];
    C* wred = reinterpret_cast<C*>(wred_raw);
    const int org[3] = {A.rlo[0] + (int)blockIdx.x * TX, A.rlo[1] + (int)blockIdx.y * TY,
                        A.rlo[2] + (int)blockIdx.z * TZ};
    using SL = SmemLayout<C, Physics<C, EQ, FLUX>::NV, ReconTraits<RC>::ghosts, DIM, TX, TY, TZ>;
    unsigned char* base = align_smem(smem_raw);
    C* su = reinterpret_cast<C*>(base);
    stage_tile_load<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, C, true>(A, org, su);
    stage_tile_compute<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, C, true>(A, org, su,
                                                                       reinterpret_cast<C*>(base + SL::halo_bytes), wred);
}

// The single-grid stage with the tile + halo staged by TMA (storage type =
// arithmetic type). The maps are kernel parameters; shared memory: halo, then
// the line buffers, which hold the L0 halo until U1 is formed.
template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH, int MINB = 1>
__global__ void __launch_bounds__(NTH, MINB) stage_kernel_tma(StageArgs A, const __grid_constant__ TmaMaps M) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned char wred_raw[(NTH / 32) * 3 * sizeof(R)];
    __shared__ __align__(8) unsigned long long bar;
    constexpr int NV = Physics<R, EQ, FLUX>::NV;
    using SL = SmemLayout<R, NV, ReconTraits<RC>::ghosts, DIM, TX, TY, TZ>;
    R* wred = reinterpret_cast<R*>(wred_raw);
    if (A.st->done) return;
    unsigned char* base = align_smem(smem_raw);
    R* su = reinterpret_cast<R*>(base);
    R* work = reinterpret_cast<R*>(base + SL::halo_bytes);
    const int org[3] = {(int)blockIdx.x * TX, (int)blockIdx.y * TY, (int)blockIdx.z * TZ};
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) tma_stage_issue<R, SL, DIM>(A, &M.in, &M.l0, org, su, work, &bar, false, A.tma_extra_tx);
    if (!tma_stage_finish<R, SL, NTH>(A, su, work, &bar, 0)) return;
    stage_tile_compute<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, R>(A, org, su, work, wred);
}

// The stage arguments of ensemble tile t (its member's buffers for the stage
// mode); false when the member's run is done.
__device__ __forceinline__ bool batch_tile_args(const BatchArgs& B, int t, StageArgs& A, int* org) {
    const int4 tile = B.tiles[t];
    StepState* st = B.states + tile.x;
    if (st->done) return false;  // the same value for every thread of the CTA
    const BatchMember& m = B.members[tile.x];
    // ensemble RK2 alternates the two state buffers instead of copying
    void* cur = st->parity ? m.v : m.u;
    void* other = st->parity ? m.u : m.v;
    A.G = m.G;
    A.st = st;
    A.gamma = B.gamma;
    A.gamma_f = B.gamma_f;
    A.mode = B.mode;
    A.periodic = B.periodic;
    A.check = 0;
    A.l0 = nullptr;
    A.copy_in = nullptr;
    A.out2 = nullptr;
    if (B.mode == MODE_L) {
        A.in = cur; A.u0 = cur; A.out = m.l;
    } else if (B.mode == MODE_RK3_S1) {
        A.in = cur; A.u0 = cur; A.l0 = m.l; A.out = other;
    } else if (B.mode == MODE_RK3_S2) {
        A.in = other; A.u0 = cur; A.out = cur; A.check = 1;
    } else {  // MODE_RK2_S1
        A.in = cur; A.u0 = cur; A.l0 = m.l; A.out = other; A.check = 1;
    }
    // the member's tensor maps: [0] u, [1] v, [2] l
    const CUtensorMap* mm = (B.maps && m.tma) ? B.maps + 3 * tile.x : nullptr;
    A.tm_in = mm ? mm + ((B.mode == MODE_RK3_S2) != (st->parity != 0) ? 1 : 0) : nullptr;
    A.tm_l0 = mm ? mm + 2 : nullptr;
    org[0] = tile.y;
    org[1] = tile.z;
    org[2] = tile.w;
    return true;
}

// Persistent ensemble stage: each CTA walks the tile list (tiles of every
// member grid, heterogeneous sizes) with stride gridDim.x. A member whose run
// is done is skipped as a whole; the per-member wave-speed maxima land in
// that member's step state (a segmented reduction), so every member gets its
// own dt. With storage type = arithmetic type the CTA runs a software
// pipeline: the next tile's halo streams into a second buffer (TMA when the
// kernel is built for it and the member has tensor maps, cp.async otherwise)
// while the current tile computes.
// Resident CTAs per SM the FP32 ensemble kernel is compiled for (register
// cap): 1280 threads, or fewer CTAs when their shared memory does not fit.
template <class C, int NTH, size_t SMEM> struct BatchMinBlocks {
    static constexpr int by_threads = 1280 / NTH > 0 ? 1280 / NTH : 1;
    static constexpr int by_smem = (int)((225 * 1024) / SMEM) > 0 ? (int)((225 * 1024) / SMEM) : 1;
    static constexpr int value =
        std::is_same<C, float>::value ? (by_threads < by_smem ? by_threads : by_smem) : 1;
};

template <class R, int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH, class C = R, bool TMA = false>
__global__ void __launch_bounds__(
    NTH, (BatchMinBlocks<C, NTH,
                         SmemLayout<C, Physics<C, EQ, FLUX>::NV, ReconTraits<RC>::ghosts, DIM, TX, TY, TZ>::pipe_bytes>::value))
    batch_stage_kernel(BatchArgs B) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned char wred_raw[(NTH / 32) * 3 * sizeof(C)];
    __shared__ __align__(8) unsigned long long bar;
    C* wred = reinterpret_cast<C*>(wred_raw);
    unsigned char* base = align_smem(smem_raw);
    const int ntiles = *B.ntiles;
    if constexpr (std::is_same<R, C>::value) {
        // shared memory: halo A, halo B, L0 halo, line buffers
        constexpr int NV = Physics<C, EQ, FLUX>::NV;
        using SL = SmemLayout<C, NV, ReconTraits<RC>::ghosts, DIM, TX, TY, TZ>;
        C* cur_h = reinterpret_cast<C*>(base);
        C* next_h = reinterpret_cast<C*>(base + SL::halo_bytes);
        C* l0h = reinterpret_cast<C*>(base + 2 * SL::halo_bytes);
        C* work = reinterpret_cast<C*>(base + 3 * SL::halo_bytes);
        if constexpr (TMA) {
            if (threadIdx.x == 0) mbar_init(&bar, 1);
            __syncthreads();
        }
        unsigned phase = 0;
        StageArgs A;
        int org[3];
        int t = blockIdx.x;
        while (t < ntiles && !batch_tile_args(B, t, A, org)) t += gridDim.x;
        if (t >= ntiles) return;
        if (TMA && A.tm_in) {
            if (threadIdx.x == 0) tma_stage_issue<R, SL, DIM>(A, A.tm_in, A.tm_l0, org, cur_h, l0h, &bar, true);
            if (!tma_stage_finish<R, SL, NTH>(A, cur_h, l0h, &bar, phase)) return;
            phase ^= 1u;
        } else {
            stage_tile_load<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, C>(A, org, cur_h);
        }
        while (true) {
            // issue the next tile's staging; only its index and kind stay
            // live across the compute phase (its arguments are rebuilt after)
            int tn = t + gridDim.x;
            bool next_tma = false;
            {
                StageArgs An;
                int orgn[3];
                while (tn < ntiles && !batch_tile_args(B, tn, An, orgn)) tn += gridDim.x;
                if (tn < ntiles) {
                    next_tma = TMA && An.tm_in != nullptr;
                    if (next_tma) {
                        if (threadIdx.x == 0)
                            tma_stage_issue<R, SL, DIM>(An, An.tm_in, An.tm_l0, orgn, next_h, l0h, &bar, true);
                    } else {
                        stage_tile_prefetch<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH>(An, orgn, next_h, l0h);
                    }
                }
            }
            stage_tile_compute<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, C>(A, org, cur_h, work, wred);
            // this thread's generic writes of the halo buffers (U1 combine,
            // edge fill) before later TMA writes into them
            if constexpr (TMA) fence_proxy_async_smem();
            __syncthreads();
            if (tn >= ntiles) break;
            batch_tile_args(B, tn, A, org);  // the member's done flag is fixed during the launch
            if (next_tma) {
                if (!tma_stage_finish<R, SL, NTH>(A, next_h, l0h, &bar, phase)) return;
                phase ^= 1u;
            } else {
                stage_tile_prefetch_finish<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH>(A, next_h, l0h);
            }
            C* tmp = cur_h;
            cur_h = next_h;
            next_h = tmp;
            t = tn;
        }
    } else {
        (void)bar;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            StageArgs A;
            int org[3];
            if (!batch_tile_args(B, t, A, org)) continue;
            stage_tile<R, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, C>(A, org, base, wred);
            __syncthreads();
        }
    }
}

// Forward-Euler update U += L0 * c in place with ghost images
// (alsfvm/src/integrator/ForwardEuler.cpp:32-51).
template <class R, int EQ>
__global__ void fe_apply_kernel(StageArgs A) {
    using Ph = Physics<R, EQ, 1>;
    constexpr int NV = Ph::NV;
    if (A.st->done) return;
    const Grid& Gd = A.G;
    const long long ncell = (long long)Gd.n[0] * Gd.n[1] * Gd.n[2];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncell) return;
    const int ix = (int)(i % Gd.n[0]);
    const int iy = (int)((i / Gd.n[0]) % Gd.n[1]);
    const int iz = (int)(i / ((long long)Gd.n[0] * Gd.n[1]));
    const R* l0 = reinterpret_cast<const R*>(A.l0);
    R* out = reinterpret_cast<R*>(A.out);
    const long long total = Gd.total;
    const long long own = gidx(Gd, ix + Gd.g[0], iy + Gd.g[1], iz + Gd.g[2]);
    const R scale = uniform_value<R>(A.st->scale, A.st->scale_f);
    R res[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) res[k] = madd(l0[k * total + own], scale, out[k * total + own]);
    if (A.check && !Ph::obeys(res, uniform_value<R>(A.gamma, A.gamma_f))) {
        if (atomicExch(&A.st->status, 1) == 0) A.st->failed_step = (int)A.st->steps + 1;
    }
    store_with_images<R, NV>(out, total, Gd, ix, iy, iz, A.periodic != 0, res);
}

}  // namespace GBFV_VARIANT_NS
}  // namespace gbfv
