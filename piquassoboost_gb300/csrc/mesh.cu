// Clements rectangular mesh: the m x m unitary of m(m-1)/2 Mach-Zehnder
// interferometers and its adjoint with respect to the m(m-1) phases.
//
// No counterpart in the reference: this is the differentiable interferometer
// in front of the batched permanent gradient (a log-likelihood of sampled
// patterns backpropagated to the mesh phases).
//
// Layer l (l = 0 .. m-1) holds the interferometers on mode pairs (i, i+1),
// i = l mod 2, l mod 2 + 2, ..., i + 1 <= m - 1; interferometer t (counted
// layer by layer, then by i) has phases (theta, phi) = (ph[2t], ph[2t+1]) and
// maps rows (i, i+1) of the running matrix X by
//     [[e^{i phi} cos theta, -sin theta], [e^{i phi} sin theta, cos theta]],
// so U = L_{m-1} ... L_1 L_0.
//
// Left multiplication leaves the columns of X independent: one warp walks
// one column through all m layers, lane p owning pair p of the layer (pairs
// of a layer are disjoint, so a layer needs only a warp barrier).  The layer
// loop is a chain of m dependent steps, so everything it reads is staged in
// shared memory first.  The coefficients are computed once per
// interferometer by a separate launch (FP64 sincos spread over the chip
// instead of repeated per column).
//
// Backward (gU = dL/dU in torch's convention for complex tensors, the
// derivative with respect to the real part plus i times that with respect to
// the imaginary part): G = gU walks back through the layers as
// G <- L_l^H G, column by column; for interferometer t with 2x2 block
// (a, b; c, d) acting on rows (i, i+1) of the previous state x,
//     g_a = sum_j G_i[j] conj(x_i[j]),  g_b = sum_j G_i[j] conj(x_{i+1}[j]),
//     g_c = sum_j G_{i+1}[j] conj(x_i[j]),  g_d = sum_j G_{i+1}[j] conj(x_{i+1}[j]),
// and dL/dp = Re(sum_k conj(g_k) dk/dp) for p in {theta, phi}.  The column
// terms are written per column and summed by a third launch in an order that
// does not depend on scheduling, so the phase gradient is deterministic.
#include <algorithm>
#include <cstdint>
#include <cstring>

#include "gbperm.h"
#include "gbperm_capi_internal.h"

namespace gbperm {

namespace {

constexpr int kMeshMax = 64;        // modes; a layer has at most 32 pairs (one warp)
constexpr int kMeshThreads = 128;   // staging threads per block; warp 0 walks the block's column

// a * conj(b)
__device__ __forceinline__ double2 zmulc(double2 a, double2 b) {
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// coefficients (a, b, c, d) of every interferometer
__global__ void mesh_coef_kernel(const double* __restrict__ ph, int nmzi, double2* __restrict__ coef) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nmzi) return;
    double st, ct, sp, cp;
    sincos(ph[2 * t], &st, &ct);
    sincos(ph[2 * t + 1], &sp, &cp);
    coef[4 * t + 0] = make_double2(cp * ct, sp * ct);
    coef[4 * t + 1] = make_double2(-st, 0.0);
    coef[4 * t + 2] = make_double2(cp * st, sp * st);
    coef[4 * t + 3] = make_double2(ct, 0.0);
}

// Forward: block j walks column j (one column per block, so the FP64 work
// of the m columns spreads over m SMs; every warp helps stage, warp 0
// walks).  The state after layer l goes to states[(j * m + l) * m + i] for
// the backward.
__global__ void __launch_bounds__(kMeshThreads) mesh_forward_kernel(const double2* __restrict__ coef, int m, int nmzi,
                                                                    double2* __restrict__ U,
                                                                    double2* __restrict__ states) {
    extern __shared__ __align__(16) double2 smem[];
    double2* s_coef = smem;                // nmzi x 4
    double2* x = smem + 4 * (size_t)nmzi;  // kMeshMax
    for (int e = threadIdx.x; e < 4 * nmzi; e += blockDim.x) s_coef[e] = coef[e];
    const int p = threadIdx.x;
    const int j = blockIdx.x;
    if (p < 32)
        for (int i = p; i < m; i += 32) x[i] = make_double2(i == j ? 1.0 : 0.0, 0.0);
    __syncthreads();
    if (p >= 32) return;  // no block barrier below
    double2* st = states + (size_t)j * m * m;
    int t0 = 0;
    for (int l = 0; l < m; ++l) {
        const int par = l & 1;
        const int np = (m - par) >> 1;
        if (p < np) {
            const int i = par + 2 * p;
            const double2* k = s_coef + 4 * (t0 + p);
            const double2 a = k[0], c = k[2];
            const double b = k[1].x, d = k[3].x;  // real entries
            const double2 xi = x[i], xi1 = x[i + 1];
            x[i] = make_double2(fma(a.x, xi.x, fma(-a.y, xi.y, b * xi1.x)), fma(a.x, xi.y, fma(a.y, xi.x, b * xi1.y)));
            x[i + 1] = make_double2(fma(c.x, xi.x, fma(-c.y, xi.y, d * xi1.x)),
                                    fma(c.x, xi.y, fma(c.y, xi.x, d * xi1.y)));
        }
        __syncwarp();
        for (int i = p; i < m; i += 32) st[(size_t)l * m + i] = x[i];
        __syncwarp();  // the copy reads rows the next layer's lanes overwrite
        t0 += np;
    }
    for (int i = p; i < m; i += 32) U[(size_t)i * m + j] = x[i];
}

// Backward: block j walks G[:, j] back through the layers with the
// coefficients and column j's layer states staged in shared memory (every
// warp stages, warp 0 walks); for interferometer t the four terms of column
// j go to part[(t * m + j) * 4 + k].
__global__ void __launch_bounds__(kMeshThreads) mesh_backward_kernel(const double2* __restrict__ coef, int m,
                                                                     int nmzi, const double2* __restrict__ states,
                                                                     const double2* __restrict__ gU,
                                                                     double2* __restrict__ part) {
    extern __shared__ __align__(16) double2 smem[];
    double2* s_coef = smem;                 // nmzi x 4
    double2* st = smem + 4 * (size_t)nmzi;  // m x m (layer, row) of column j
    double2* g = st + (size_t)m * m;        // kMeshMax
    const int j = blockIdx.x;
    for (int e = threadIdx.x; e < 4 * nmzi; e += blockDim.x) s_coef[e] = coef[e];
    const double2* src = states + (size_t)j * m * m;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) st[e] = src[e];
    const int p = threadIdx.x;
    if (p < 32)
        for (int i = p; i < m; i += 32) g[i] = gU[(size_t)i * m + j];
    __syncthreads();
    if (p >= 32) return;  // no block barrier below
    int t0 = nmzi;
    for (int l = m - 1; l >= 0; --l) {
        const int par = l & 1;
        const int np = (m - par) >> 1;
        t0 -= np;
        if (p < np) {
            const int i = par + 2 * p;
            const int t = t0 + p;
            double2 xi, xi1;
            if (l > 0) {
                xi = st[(size_t)(l - 1) * m + i];
                xi1 = st[(size_t)(l - 1) * m + i + 1];
            } else {
                xi = make_double2(i == j ? 1.0 : 0.0, 0.0);
                xi1 = make_double2(i + 1 == j ? 1.0 : 0.0, 0.0);
            }
            const double2 gi = g[i], gi1 = g[i + 1];
            double2* q = part + ((size_t)t * m + j) * 4;
            q[0] = zmulc(gi, xi);
            q[1] = zmulc(gi, xi1);
            q[2] = zmulc(gi1, xi);
            q[3] = zmulc(gi1, xi1);
            const double2* k = s_coef + 4 * t;
            const double2 a = k[0], c = k[2];
            const double b = k[1].x, d = k[3].x;  // real entries
            // rows (i, i+1) <- L^H (gi, gi1) = (conj(a) gi + conj(c) gi1, b gi + d gi1)
            g[i] = make_double2(fma(a.x, gi.x, fma(a.y, gi.y, fma(c.x, gi1.x, c.y * gi1.y))),
                                fma(a.x, gi.y, fma(-a.y, gi.x, fma(c.x, gi1.y, -c.y * gi1.x))));
            g[i + 1] = make_double2(fma(b, gi.x, d * gi1.x), fma(b, gi.y, d * gi1.y));
        }
        __syncwarp();
    }
}

// Warp per interferometer: lane j mod 32 sums the terms of columns j, then a
// butterfly (fl addition commutes, so all lanes agree and nothing depends on
// scheduling); lane 0 maps the four sums to the two phases.
__global__ void mesh_phase_grad_kernel(const double* __restrict__ ph, int m, int nmzi,
                                       const double2* __restrict__ part, double* __restrict__ gph) {
    const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (t >= nmzi) return;  // warp-uniform
    double v[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int j = lane; j < m; j += 32) {
        const double2* q = part + ((size_t)t * m + j) * 4;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double2 z = q[k];
            v[2 * k] += z.x;
            v[2 * k + 1] += z.y;
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    if (lane != 0) return;
    double st, ct, sp, cp;
    sincos(ph[2 * t], &st, &ct);
    sincos(ph[2 * t + 1], &sp, &cp);
    // Re(conj(g) z) = g.x z.x + g.y z.y with g = (v[2k], v[2k+1])
    // da/dtheta = -e^{i phi} sin, db/dtheta = -cos, dc/dtheta = e^{i phi} cos, dd/dtheta = -sin
    const double dth = v[0] * (-cp * st) + v[1] * (-sp * st) + v[2] * (-ct) + v[4] * (cp * ct) + v[5] * (sp * ct) +
                       v[6] * (-st);
    // da/dphi = i e^{i phi} cos, dc/dphi = i e^{i phi} sin
    const double dph = v[0] * (-sp * ct) + v[1] * (cp * ct) + v[4] * (-sp * st) + v[5] * (cp * st);
    gph[2 * t] = dth;
    gph[2 * t + 1] = dph;
}

struct MeshWs {
    size_t coef = 0, states = 0, part = 0, total = 0;
};

MeshWs mesh_ws(int64_t m) {
    MeshWs w;
    const size_t nmzi = (size_t)(m * (m - 1) / 2);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += align_up(bytes, 256);
        return o;
    };
    w.coef = take(nmzi * 4 * sizeof(double2));
    w.states = take((size_t)m * m * m * sizeof(double2));
    w.part = take(nmzi * (size_t)m * 4 * sizeof(double2));
    w.total = off;
    return w;
}

int mesh_check(const char* who, int64_t m, const void* ws, size_t ws_bytes) {
    if (m < 1 || m > kMeshMax) return fail(GBPERM_ERR_TOO_LARGE, std::string(who) + ": modes must be in 1..64");
    if (!ws) return fail(GBPERM_ERR_ARG, std::string(who) + ": null workspace");
    if (reinterpret_cast<uintptr_t>(ws) % 256 != 0)
        return fail(GBPERM_ERR_ARG, std::string(who) + ": workspace must be 256-byte aligned");
    if (ws_bytes < mesh_ws(m).total) return fail(GBPERM_ERR_ARG, std::string(who) + ": workspace too small");
    return GBPERM_OK;
}

}  // namespace

}  // namespace gbperm

using namespace gbperm;

extern "C" size_t gbperm_mesh_workspace_size(int64_t m) {
    if (m < 1 || m > kMeshMax) return 0;
    return mesh_ws(m).total;
}

extern "C" int gbperm_mesh_unitary_dev(const void* d_phases, int64_t m, void* d_U, void* workspace,
                                       size_t workspace_bytes, void* stream) {
    int rc = mesh_check("gbperm_mesh_unitary_dev", m, workspace, workspace_bytes);
    if (rc) return rc;
    if (!d_U || (m > 1 && !d_phases)) return fail(GBPERM_ERR_ARG, "gbperm_mesh_unitary_dev: null pointer");
    if (reinterpret_cast<uintptr_t>(d_U) % 16 != 0 || reinterpret_cast<uintptr_t>(d_phases) % 8 != 0)
        return fail(GBPERM_ERR_ARG, "gbperm_mesh_unitary_dev: misaligned pointer");
    const MeshWs w = mesh_ws(m);
    char* base = static_cast<char*>(workspace);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nmzi = (int)(m * (m - 1) / 2);
    double2* coef = reinterpret_cast<double2*>(base + w.coef);
    if (nmzi > 0) mesh_coef_kernel<<<(nmzi + 127) / 128, 128, 0, st>>>(static_cast<const double*>(d_phases), nmzi, coef);
    const size_t smem = ((size_t)nmzi * 4 + kMeshMax) * sizeof(double2);
    cudaError_t e = allow_max_dynamic_smem((const void*)mesh_forward_kernel);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_mesh_unitary_dev: shared memory");
    mesh_forward_kernel<<<(int)m, kMeshThreads, smem, st>>>(coef, (int)m, nmzi, static_cast<double2*>(d_U),
                                                            reinterpret_cast<double2*>(base + w.states));
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_mesh_unitary_dev: launch");
    return GBPERM_OK;
}

extern "C" int gbperm_mesh_unitary_backward_dev(const void* d_phases, int64_t m, const void* d_gU, void* d_gphases,
                                                void* workspace, size_t workspace_bytes, void* stream) {
    int rc = mesh_check("gbperm_mesh_unitary_backward_dev", m, workspace, workspace_bytes);
    if (rc) return rc;
    const int nmzi = (int)(m * (m - 1) / 2);
    if (nmzi == 0) return GBPERM_OK;
    if (!d_phases || !d_gU || !d_gphases)
        return fail(GBPERM_ERR_ARG, "gbperm_mesh_unitary_backward_dev: null pointer");
    if (reinterpret_cast<uintptr_t>(d_gU) % 16 != 0 || reinterpret_cast<uintptr_t>(d_phases) % 8 != 0 ||
        reinterpret_cast<uintptr_t>(d_gphases) % 8 != 0)
        return fail(GBPERM_ERR_ARG, "gbperm_mesh_unitary_backward_dev: misaligned pointer");
    const MeshWs w = mesh_ws(m);
    char* base = static_cast<char*>(workspace);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double2* part = reinterpret_cast<double2*>(base + w.part);
    const size_t smem = ((size_t)nmzi * 4 + (size_t)m * m + kMeshMax) * sizeof(double2);
    cudaError_t e = allow_max_dynamic_smem((const void*)mesh_backward_kernel);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_mesh_unitary_backward_dev: shared memory");
    mesh_backward_kernel<<<(int)m, kMeshThreads, smem, st>>>(reinterpret_cast<const double2*>(base + w.coef), (int)m,
                                                             nmzi, reinterpret_cast<const double2*>(base + w.states),
                                                             static_cast<const double2*>(d_gU), part);
    const int wpb = 4;  // warps (interferometers) per block
    mesh_phase_grad_kernel<<<(nmzi + wpb - 1) / wpb, 32 * wpb, 0, st>>>(static_cast<const double*>(d_phases), (int)m,
                                                                         nmzi, part, static_cast<double*>(d_gphases));
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_mesh_unitary_backward_dev: launch");
    return GBPERM_OK;
}
