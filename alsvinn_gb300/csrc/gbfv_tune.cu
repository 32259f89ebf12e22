// Host support of the TMA staging and the autotuner: tensor-map encoding of
// the padded SoA state arrays (cuTensorMapEncodeTiled, reached through the
// runtime's driver entry-point query so the library does not link libcuda),
// the process-wide cache of autotuned choices and the GBFV_AUTOTUNE switch.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "fv_tma.cuh"
#include "gbfv_internal.h"

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

std::mutex g_tune_mu;
std::map<std::string, int>& tune_cache() {
    static std::map<std::string, int> m;
    return m;
}

}  // namespace

bool gbfv_encode_state_map(CUtensorMap* map, const void* base, const gbfv::Grid& G, int nvar, int elem, int hx,
                           int hy, int hz) {
    if (!map || !base || (elem != 4 && elem != 8) || nvar < 1 || nvar > 256) return false;
    const int dim = G.dim;
    if (dim < 1 || dim > 3) return false;
    // TMA rules: 16-byte aligned base, strides and box rows multiples of 16
    // bytes, box extents 1..256
    if (reinterpret_cast<std::uintptr_t>(base) % 16 != 0) return false;
    if (((long long)G.t[0] * elem) % 16 != 0) return false;
    if (((long long)hx * elem) % 16 != 0) return false;
    const int box[3] = {hx, hy, hz};
    cuuint64_t dims[4], strides[3];
    cuuint32_t boxd[4], es[4];
    int rank = 0;
    for (int d = 0; d < dim; ++d) {
        if (box[d] < 1 || box[d] > 256) return false;
        dims[rank] = (cuuint64_t)G.t[d];
        boxd[rank] = (cuuint32_t)box[d];
        es[rank] = 1;
        ++rank;
    }
    dims[rank] = (cuuint64_t)nvar;
    boxd[rank] = (cuuint32_t)nvar;
    es[rank] = 1;
    ++rank;
    // byte strides of dimensions 1 .. rank-1: rows, planes, then variables
    long long row = elem;
    int k = 0;
    for (int d = 0; d + 1 < dim; ++d) {
        row *= G.t[d];
        strides[k++] = (cuuint64_t)row;
    }
    strides[k++] = (cuuint64_t)(G.total * elem);
    for (int i = 0; i < k; ++i)
        if (strides[i] % 16 != 0 || strides[i] >= (1ull << 40)) return false;
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) return false;
    CUtensorMap m;
    const CUresult r =
        fn(&m, elem == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank,
           const_cast<void*>(base), dims, strides, boxd, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    *map = m;
    return true;
}

int gbfv_autotune_enabled() {
    const char* v = std::getenv("GBFV_AUTOTUNE");
    return !(v && std::strcmp(v, "0") == 0);
}

bool gbfv_tune_cache_get(const char* key, int* cand) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = tune_cache().find(key);
    if (it == tune_cache().end()) return false;
    *cand = it->second;
    return true;
}

void gbfv_tune_cache_put(const char* key, int cand) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_cache()[key] = cand;
}
