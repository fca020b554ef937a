// Element barycentres of a mesh, on the device: the points coupe's mesh-part
// partitions (tools/lib/lib.rs:511-539, `barycentres`).  For one block of
// elements with the same node count k, each barycentre is the sum of its k
// node coordinates taken in the element's node order, starting from 0.0,
// divided by k: coupe's arithmetic, so the points are bit-identical.  One
// thread per element; the node lists are read once (k x 8 B per element) and
// the node coordinates gathered (neighbouring elements share nodes, which
// L2 keeps).  A node index >= the node count is an error (coupe's
// mesh.node(i) panics).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>

#include "engine.h"
#include "kernels.cuh"

namespace cg {

namespace {

struct MeshScratch {
    unsigned long long first_bad;  // smallest element index with a bad node index
    uint32_t flags;
    uint32_t pad;
};

template <int D, int K>
__global__ void __launch_bounds__(BLOCK) k_barycentres(const double *__restrict__ coords, uint64_t n_nodes,
                                                       const uint64_t *__restrict__ nodes, uint64_t n_el,
                                                       double *__restrict__ out, MeshScratch *sc) {
    for (uint64_t e = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; e < n_el; e += (uint64_t)gridDim.x * BLOCK) {
        uint64_t v[K];
#pragma unroll
        for (int j = 0; j < K; ++j) v[j] = __ldg(nodes + e * K + j);
        double acc[D];
#pragma unroll
        for (int d = 0; d < D; ++d) acc[d] = 0.0;
        bool ok = true;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            if (v[j] >= n_nodes) {
                ok = false;
                continue;
            }
#pragma unroll
            for (int d = 0; d < D; ++d) acc[d] = __dadd_rn(acc[d], __ldg(coords + v[j] * D + d));
        }
        if (!ok) {
            atomicOr(&sc->flags, 1u);
            atomicMin(&sc->first_bad, (unsigned long long)e);
        }
#pragma unroll
        for (int d = 0; d < D; ++d) out[e * D + d] = acc[d] / (double)K;
    }
}

template <int D, int K>
int launch_bary(DevCtx &C, const double *coords, uint64_t n_nodes, const uint64_t *nodes, uint64_t n_el,
                double *out, MeshScratch *sc, cudaStream_t s, std::string *err) {
    const unsigned grid = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((n_el + BLOCK - 1) / BLOCK, (uint64_t)C.sms * 8));
    C.prof.begin(KID_BARY, n_el * (K * 8 + D * 8) + n_nodes * D * 8, s);
    k_barycentres<D, K><<<grid, BLOCK, 0, s>>>(coords, n_nodes, nodes, n_el, out, sc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "k_barycentres", err);
    C.prof.end(s);
    return COUPE_ERR_OK;
}

}  // namespace

int barycentres(DevCtx &C, int dim, const double *d_coords, uint64_t n_nodes, uint64_t k, const uint64_t *d_nodes,
                uint64_t n_el, double *d_out, cudaStream_t stream, std::string *err) {
    cudaStream_t s = stream ? stream : C.stream;
    if (n_el == 0) return COUPE_ERR_OK;
    int rc = ensure_workspace(C, 256, err);
    if (rc != COUPE_ERR_OK) return rc;
    MeshScratch *sc = (MeshScratch *)C.ws;
    MeshScratch init{};
    init.first_bad = ~0ull;
    cudaError_t e = cudaMemcpyAsync(sc, &init, sizeof(init), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "barycentre set-up", err);
#define CG_BARY(DD, KK) \
    if (dim == DD && k == KK) rc = launch_bary<DD, KK>(C, d_coords, n_nodes, d_nodes, n_el, d_out, sc, s, err)
    rc = -1;
    CG_BARY(2, 2); else CG_BARY(2, 3); else CG_BARY(2, 4); else CG_BARY(2, 8);
    else CG_BARY(3, 2); else CG_BARY(3, 3); else CG_BARY(3, 4); else CG_BARY(3, 8);
#undef CG_BARY
    if (rc == -1) {
        if (err) *err = "elements of 2, 3, 4 or 8 nodes in dimension 2 or 3";
        return dim == 2 || dim == 3 ? COUPE_ERR_BAD_TYPE : COUPE_ERR_BAD_DIMENSION;
    }
    if (rc != COUPE_ERR_OK) return rc;
    MeshScratch hs;
    if ((e = cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "barycentre read-back", err);
    C.prof.resolve();
    if (hs.flags) {
        if (err) *err = "node index out of range in element " + std::to_string(hs.first_bad);
        return COUPE_ERR_BAD_TYPE;
    }
    return COUPE_ERR_OK;
}

}  // namespace cg
