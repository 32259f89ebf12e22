// Kernel instantiations for one arithmetic variant and one equation. This file
// is compiled twice per (FV_VARIANT, FV_EQ) pair (FV_PART 0: every scheme's
// default stage kernels and the operator-level kernels; FV_PART 1: the
// autotuning candidates), so the units build in parallel. Every variant is
// built with -fmad=false: no multiply-add is contracted unless the source
// writes the FMA, so every candidate of a scheme rounds alike; the exact
// variant (FV_EXACT) writes none and follows the reference's operation order.
//   FV_VARIANT: 0 fp64, 1 fp64 exact, 2 fp32 state and arithmetic,
//               3 fp64 state with double-float arithmetic on the FP32 pipes
//   FV_EQ:      0 burgers, 1 euler1, 2 euler2, 3 euler3
#define FV_NS_CAT2(a, b) a##b
#define FV_NS_CAT(a, b) FV_NS_CAT2(a, b)
#define GBFV_VARIANT_NS FV_NS_CAT(v, FV_VARIANT)
#include "fv_registry.h"
#include "fv_stage.cuh"

#ifndef FV_VARIANT
#error "FV_VARIANT must be defined"
#endif
#ifndef FV_EQ
#error "FV_EQ must be defined"
#endif

#if FV_VARIANT == 2
typedef float Real;
#else
typedef double Real;
#endif
// arithmetic of reconstruction and fluxes: the storage type, or double-float
// on the FP32 pipes for the FP64 state of variant 3
#if FV_VARIANT == 3
typedef gbfv::dfloat Compute;
#else
typedef Real Compute;
#endif

#ifndef FV_PART
#define FV_PART 0  // 0: default candidates and the other launchers, 1: autotuning candidates, 2: region kernels
#endif

#define FV_CAT2(a, b, c, d) a##b##c##d
#define FV_CAT(a, b, c, d) FV_CAT2(a, b, c, d)
#define FV_REGISTER_FN FV_CAT(gbfv_register_v, FV_VARIANT, _e, FV_EQ)
#define FV_TUNE_FN FV_CAT(gbfv_tune_v, FV_VARIANT, _e, FV_EQ)
#define FV_REGION_FN FV_CAT(gbfv_region_v, FV_VARIANT, _e, FV_EQ)

namespace gbfv {
namespace GBFV_VARIANT_NS {

// One candidate configuration of a scheme's stage kernels (tile TX x TY x TZ,
// NTH threads, TMA or plain halo staging) and its launchers.
template <int EQ, int FLUX, int RC, int DIM, int TX, int TY, int TZ, int NTH, bool TMA, int MINB = 1>
struct Cand {
    static constexpr int NV = Physics<Real, EQ, FLUX>::NV;
    static constexpr int G = ReconTraits<RC>::ghosts;
    using SL = SmemLayout<Compute, NV, G, DIM, TX, TY, TZ>;
    static constexpr bool kSame = std::is_same<Real, Compute>::value;
    static_assert(!TMA || kSame, "TMA staging copies the storage type into shared memory");
    static_assert(!TMA || (SL::HX * sizeof(Real)) % 16 == 0, "a TMA box row must be a multiple of 16 bytes");
    static_assert(!TMA || (TX * sizeof(Real)) % 16 == 0, "TMA box origins must be 16-byte aligned along x");
    static_assert(!TMA || (SL::HX <= 256 && SL::HY <= 256 && SL::HZ <= 256), "TMA box extents are at most 256");
    static constexpr size_t stage_smem = TMA ? SL::tma_bytes : SL::bytes;
    // the ensemble kernel pipelines the halo when storage and arithmetic types agree
    static constexpr size_t batch_smem = kSame ? SL::pipe_bytes : SL::bytes;

    static int launch(const StageArgs& a, const TmaMaps* maps, cudaStream_t s) {
        const dim3 grid((a.G.n[0] + TX - 1) / TX, (a.G.n[1] + TY - 1) / TY, (a.G.n[2] + TZ - 1) / TZ);
        if constexpr (TMA) {
            if (!maps) return (int)cudaErrorInvalidValue;
            auto k = stage_kernel_tma<Real, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, MINB>;
            static int configured = 0;
            if (!configured) {
                cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage_smem);
                if (e != cudaSuccess) return (int)e;
                configured = 1;
            }
            k<<<grid, NTH, stage_smem, s>>>(a, *maps);
        } else {
            auto k = stage_kernel<Real, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, Compute, MINB>;
            static int configured = 0;
            if (!configured) {
                cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage_smem);
                if (e != cudaSuccess) return (int)e;
                configured = 1;
            }
            k<<<grid, NTH, stage_smem, s>>>(a);
        }
        return (int)cudaGetLastError();
    }

    // the region kernel (operator on part of the grid): per-thread loads
    static int launch_region(const StageArgs& a, cudaStream_t s) {
        static_assert(!TMA, "the region kernel stages its halo with per-thread loads");
        const dim3 grid((a.rhi[0] - a.rlo[0] + TX - 1) / TX, (a.rhi[1] - a.rlo[1] + TY - 1) / TY,
                        (a.rhi[2] - a.rlo[2] + TZ - 1) / TZ);
        auto k = region_kernel<Real, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, Compute>;
        static int configured = 0;
        if (!configured) {
            cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SL::bytes);
            if (e != cudaSuccess) return (int)e;
            configured = 1;
        }
        k<<<grid, NTH, SL::bytes, s>>>(a);
        return (int)cudaGetLastError();
    }

    static int launch_batch(const BatchArgs& a, int ctas, cudaStream_t s) {
        auto k = batch_stage_kernel<Real, EQ, FLUX, RC, DIM, TX, TY, TZ, NTH, Compute, TMA>;
        static int resident = 0;
        if (!resident) {
            cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)batch_smem);
            if (e != cudaSuccess) return (int)e;
            int per_sm = 0, dev = 0, sms = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, NTH, batch_smem);
            if (e == cudaSuccess) e = cudaGetDevice(&dev);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return (int)e;
            resident = (per_sm > 0 ? per_sm : 1) * sms;
        }
        k<<<ctas > 0 ? ctas : resident, NTH, batch_smem, s>>>(a);
        return (int)cudaGetLastError();
    }

    static void add(Registry& R, int flux, int rc) {
        constexpr int V = FV_VARIANT, E = EQ;
        int& n = R.ncand[V][E][flux][rc][DIM - 1];
        if (n >= kMaxCandidates) return;
        StageCandidate& c = R.cand[V][E][flux][rc][DIM - 1][n++];
        c.stage = &launch;
        c.batch = &launch_batch;
        c.tile[0] = TX;
        c.tile[1] = TY;
        c.tile[2] = TZ;
        c.threads = NTH;
        c.tma = TMA ? 1 : 0;
        c.halo[0] = SL::HX;
        c.halo[1] = SL::HY;
        c.halo[2] = SL::HZ;
        c.nv = NV;
        c.min_blocks = MINB;
    }
};

template <int EQ>
static int launch_apply(const StageArgs& a, cudaStream_t s) {
    const long long ncell = (long long)a.G.n[0] * a.G.n[1] * a.G.n[2];
    const int bs = 256;
    fe_apply_kernel<Real, EQ><<<(unsigned)((ncell + bs - 1) / bs), bs, 0, s>>>(a);
    return (int)cudaGetLastError();
}

// Standalone reconstruction in one direction, global memory in and out.
template <int NV, int RC>
__global__ void recon_kernel(ReconArgs A) {
    const Grid& G = A.G;
    constexpr int g = ReconTraits<RC>::ghosts;
    (void)g;
    const int d = A.dir;
    int lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        // "none" copies every cell and ignores the range (NoReconstruction.cpp:52-64)
        lo[k] = RC == RC_NONE ? 0 : G.g[k] - (k == d) + A.start[k];
        hi[k] = RC == RC_NONE ? G.t[k] : G.t[k] - G.g[k] + (k == d) + A.end[k];
    }
    if (hi[0] <= lo[0] || hi[1] <= lo[1] || hi[2] <= lo[2]) return;
    const long long ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ex * ey * ez) return;
    const int x = lo[0] + (int)(i % ex);
    const int y = lo[1] + (int)((i / ex) % ey);
    const int z = lo[2] + (int)(i / (ex * ey));
    const long long gi = gidx(G, x, y, z);
    const int ds = d == 0 ? 1 : (d == 1 ? G.t[0] : G.t[0] * G.t[1]);
    const Real* in = reinterpret_cast<const Real*>(A.in);
    Real l[NV], r[NV];
    reconstruct_cell<Real, NV, RC>(in + gi, (int)G.total, ds, l, r, (Real)A.gamma);
    Real* L = reinterpret_cast<Real*>(A.left);
    Real* Rr = reinterpret_cast<Real*>(A.right);
    for (int k = 0; k < NV; ++k) {
        L[k * G.total + gi] = l[k];
        Rr[k * G.total + gi] = r[k];
    }
}

template <int EQ, int RC>
static int launch_recon(const ReconArgs& a, cudaStream_t s) {
    constexpr int NV = EQ == 0 ? 1 : EQ + 2;
    long long cnt = 1;
    for (int k = 0; k < 3; ++k) {
        const long long e = RC == RC_NONE ? a.G.t[k] : (a.G.t[k] - 2 * a.G.g[k] + 2 * (k == a.dir) + a.end[k] - a.start[k]);
        cnt *= e > 0 ? e : 0;
    }
    if (cnt == 0) return (int)cudaGetLastError();
    const int bs = 256;
    recon_kernel<NV, RC><<<(unsigned)((cnt + bs - 1) / bs), bs, 0, s>>>(a);
    return (int)cudaGetLastError();
}

template <int EQ>
__global__ void check_kernel(CheckArgs A) {
    constexpr int NV = EQ == 0 ? 1 : EQ + 2;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.G.total) return;
    const Real* in = reinterpret_cast<const Real*>(A.in);
    Real c[NV];
    for (int k = 0; k < NV; ++k) c[k] = in[k * A.G.total + i];
    if (!Physics<Real, EQ, 1>::obeys(c, (Real)A.gamma)) *A.flag = 0;
}

template <int EQ>
static int launch_check(const CheckArgs& a, cudaStream_t s) {
    const int bs = 256;
    check_kernel<EQ><<<(unsigned)((a.G.total + bs - 1) / bs), bs, 0, s>>>(a);
    return (int)cudaGetLastError();
}

#if FV_PART == 0
// The default candidate of a scheme: the variant's tile shape, plain loads;
// in 2D compiled for three resident CTAs per SM (an 80-register cap: the
// uncapped FP64 kernels used up to 95 registers, two CTAs per SM). The 3D
// kernels stay uncapped: at 80 registers they spill hundreds of bytes.
template <int FLUX, int RC, int DIM>
static void reg_one(Registry& R) {
    using TS = TileShape<DIM, FV_VARIANT>;
    Cand<FV_EQ, FLUX, RC, DIM, TS::X, TS::Y, TS::Z, TS::THREADS, false, (DIM == 2 ? 3 : 1)>::add(R, FLUX, RC);
}

// Every reconstruction for one flux in one dimension. The double-float
// variant covers the WENO / ENO reconstructions only (its stage kernels are
// the slowest to compile).
template <int FLUX, int DIM>
static void reg_dim(Registry& R) {
    reg_one<FLUX, RC_NONE, DIM>(R);
    reg_one<FLUX, RC_WENO2, DIM>(R);
    reg_one<FLUX, RC_ENO2, DIM>(R);
    reg_one<FLUX, RC_ENO3, DIM>(R);
    reg_one<FLUX, RC_ENO4, DIM>(R);
#if FV_VARIANT != 3
    reg_one<FLUX, RC_MC, DIM>(R);
    reg_one<FLUX, RC_MM, DIM>(R);
#if FV_EQ != 0
    reg_one<FLUX, RC_WENOF2, DIM>(R);
#endif
#endif
}
#elif FV_PART == 2
// The region kernels (the operator on part of the grid, for the
// reference's NumericalFlux::computeFlux with start / end) of every scheme
// with the default candidate's tile; their own translation units so they
// compile in parallel with the stage kernels.
template <int FLUX, int RC, int DIM>
static void reg_region_one(Registry& R) {
    using TS = TileShape<DIM, FV_VARIANT>;
    using C0 = Cand<FV_EQ, FLUX, RC, DIM, TS::X, TS::Y, TS::Z, TS::THREADS, false, (DIM == 2 ? 3 : 1)>;
    R.region[FV_VARIANT][FV_EQ][FLUX][RC][DIM - 1] = &C0::launch_region;
}

// the schemes reg_dim registers (the double-float variant: the WENO / ENO
// reconstructions with HLL, HLL3 and Godunov)
template <int FLUX, int DIM>
static void reg_region_dim(Registry& R) {
    reg_region_one<FLUX, RC_NONE, DIM>(R);
    reg_region_one<FLUX, RC_WENO2, DIM>(R);
    reg_region_one<FLUX, RC_ENO2, DIM>(R);
    reg_region_one<FLUX, RC_ENO3, DIM>(R);
    reg_region_one<FLUX, RC_ENO4, DIM>(R);
#if FV_VARIANT != 3
    reg_region_one<FLUX, RC_MC, DIM>(R);
    reg_region_one<FLUX, RC_MM, DIM>(R);
#if FV_EQ != 0
    reg_region_one<FLUX, RC_WENOF2, DIM>(R);
#endif
#endif
}
#else
// Autotuning candidates of the tuned schemes (WENO2 with HLL3 for Euler in
// its own dimension, WENO2 with Godunov for 1D Burgers): TMA staging of the
// default tile, taller / wider tiles with two cells per thread and a square
// tile; the 32 x 8, 16 x 16 and one 32 x 16 configuration are compiled for
// three resident CTAs per SM (a register cap: more warps for the FP64 pipe's
// latency); 1D adds narrower tiles, which give small grids more CTAs. Every
// candidate computes the same values in the same order per cell (the tile
// only changes which CTA computes a cell), so the states are bit-identical.
#if FV_VARIANT == 3
// The double-float variant stages through registers (FP64 -> double-float
// pairs), so its candidates use per-thread loads: the default 16 x 12 tile
// capped for four resident CTAs per SM, and 32 x 16 / 32 x 8 tiles for three
// (2D; its kernels are barrier-bound and gain from more resident warps).
template <int FLUX, int DIM>
static void reg_tuned(Registry& R) {
    constexpr int E = FV_EQ, RC = RC_WENO2;
    if constexpr (DIM == 2) {
        Cand<E, FLUX, RC, 2, 16, 12, 1, 256, false, 4>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 2, 32, 16, 1, 256, false, 3>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 2, 32, 8, 1, 256, false, 3>::add(R, FLUX, RC);
    }
    (void)R;
}
#else
template <int FLUX, int DIM>
static void reg_tuned(Registry& R) {
    constexpr int E = FV_EQ, RC = RC_WENO2;
    if constexpr (DIM == 1) {
        // threads >= tile + 2: reconstructions and faces in one pass
        Cand<E, FLUX, RC, 1, 128, 1, 1, 160, true>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 1, 64, 1, 1, 96, true>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 1, 32, 1, 1, 64, true>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 1, 240, 1, 1, 256, true>::add(R, FLUX, RC);
    } else if constexpr (DIM == 2) {
        Cand<E, FLUX, RC, 2, 32, 8, 1, 256, true, 3>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 2, 32, 16, 1, 256, true>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 2, 16, 16, 1, 256, true, 3>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 2, 64, 8, 1, 256, true>::add(R, FLUX, RC);
        // 32 x 16 compiled for three resident CTAs per SM (register cap)
        Cand<E, FLUX, RC, 2, 32, 16, 1, 256, true, 3>::add(R, FLUX, RC);
        // the same with per-thread loads: the first stage of an in-place
        // host step reads mapped host memory, which TMA does not stage
        Cand<E, FLUX, RC, 2, 32, 16, 1, 256, false, 3>::add(R, FLUX, RC);
    } else {
        Cand<E, FLUX, RC, 3, 8, 8, 4, 256, true>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 3, 16, 8, 4, 256, true>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 3, 8, 8, 8, 256, true>::add(R, FLUX, RC);
        Cand<E, FLUX, RC, 3, 16, 16, 2, 256, true>::add(R, FLUX, RC);
        // the default tile on 384 threads (its 320 / 320 / 384 reconstructions
        // and 288 / 288 / 320 faces per direction in one pass), two CTAs per SM
        Cand<E, FLUX, RC, 3, 8, 8, 4, 384, false, 2>::add(R, FLUX, RC);
    }
}
#endif
#endif

}  // namespace GBFV_VARIANT_NS
}  // namespace gbfv

#if FV_PART == 0
extern "C" void FV_REGISTER_FN(gbfv::Registry* R) {
    using namespace gbfv;
    using namespace gbfv::GBFV_VARIANT_NS;
    constexpr int V = FV_VARIANT, E = FV_EQ;
#if FV_EQ == 0
    reg_dim<FL_GODUNOV, 1>(*R);
    reg_dim<FL_GODUNOV, 2>(*R);
    reg_dim<FL_GODUNOV, 3>(*R);
#if FV_VARIANT != 3
    reg_dim<FL_CENTRAL, 1>(*R);
    reg_dim<FL_CENTRAL, 2>(*R);
    reg_dim<FL_CENTRAL, 3>(*R);
    reg_dim<FL_RUSANOV, 1>(*R);
    reg_dim<FL_RUSANOV, 2>(*R);
    reg_dim<FL_RUSANOV, 3>(*R);
    reg_dim<FL_ROE, 1>(*R);
    reg_dim<FL_ROE, 2>(*R);
    reg_dim<FL_ROE, 3>(*R);
#endif
#else
    reg_dim<FL_HLL, FV_EQ>(*R);
    reg_dim<FL_HLL3, FV_EQ>(*R);
#if FV_VARIANT != 3
    reg_dim<FL_CENTRAL, FV_EQ>(*R);
#endif
#endif
    R->apply[V][E] = &launch_apply<E>;
    R->check[V][E] = &launch_check<E>;
    R->recon[V][E][RC_NONE] = &launch_recon<E, RC_NONE>;
    R->recon[V][E][RC_WENO2] = &launch_recon<E, RC_WENO2>;
    R->recon[V][E][RC_ENO2] = &launch_recon<E, RC_ENO2>;
    R->recon[V][E][RC_ENO3] = &launch_recon<E, RC_ENO3>;
    R->recon[V][E][RC_ENO4] = &launch_recon<E, RC_ENO4>;
    R->recon[V][E][RC_MC] = &launch_recon<E, RC_MC>;
    R->recon[V][E][RC_MM] = &launch_recon<E, RC_MM>;
#if FV_EQ != 0
    R->recon[V][E][RC_WENOF2] = &launch_recon<E, RC_WENOF2>;
#endif
}
#elif FV_PART == 2
extern "C" void FV_REGION_FN(gbfv::Registry* R) {
    using namespace gbfv;
    using namespace gbfv::GBFV_VARIANT_NS;
#if FV_EQ == 0
    reg_region_dim<FL_GODUNOV, 1>(*R);
    reg_region_dim<FL_GODUNOV, 2>(*R);
    reg_region_dim<FL_GODUNOV, 3>(*R);
#if FV_VARIANT != 3
    reg_region_dim<FL_CENTRAL, 1>(*R);
    reg_region_dim<FL_CENTRAL, 2>(*R);
    reg_region_dim<FL_CENTRAL, 3>(*R);
    reg_region_dim<FL_RUSANOV, 1>(*R);
    reg_region_dim<FL_RUSANOV, 2>(*R);
    reg_region_dim<FL_RUSANOV, 3>(*R);
    reg_region_dim<FL_ROE, 1>(*R);
    reg_region_dim<FL_ROE, 2>(*R);
    reg_region_dim<FL_ROE, 3>(*R);
#endif
#else
    reg_region_dim<FL_HLL, FV_EQ>(*R);
    reg_region_dim<FL_HLL3, FV_EQ>(*R);
#if FV_VARIANT != 3
    reg_region_dim<FL_CENTRAL, FV_EQ>(*R);
#endif
#endif
}
#else
// Runs after the default registration (candidate 0 first).
extern "C" void FV_TUNE_FN(gbfv::Registry* R) {
    using namespace gbfv;
    using namespace gbfv::GBFV_VARIANT_NS;
#if FV_EQ == 0
    reg_tuned<FL_GODUNOV, 1>(*R);
#else
    reg_tuned<FL_HLL3, FV_EQ>(*R);
#endif
}
#endif
