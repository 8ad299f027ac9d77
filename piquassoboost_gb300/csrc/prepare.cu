// Fixed-point preparation of one matrix on the device (see gbperm_internal.h).
#include "gbperm_internal.h"

namespace gbperm {

namespace {

__global__ void prepare_kernel(PrepArgs p) {
    __shared__ int s_e[64];
    for (int j = threadIdx.x; j < p.cols; j += blockDim.x) {
        double br = 0.0, bi = 0.0;
        for (int i = 0; i < p.rows; ++i) {
            double2 a = p.A[(long long)i * p.ld + j];
            double w = p.row_w ? (double)p.row_w[i] : 1.0;
            br += w * fabs(a.x);
            bi += w * fabs(a.y);
        }
        // a little headroom so that rounding in the bound never lets a sum
        // reach 2^62 in fixed point
        double b = fmax(br, bi) * (1.0 + 1e-12);
        int e = 0;
        if (b > 0.0) frexp(b, &e);
        s_e[j] = e;
        for (int i = 0; i < p.rows; ++i) {
            double2 a = p.A[(long long)i * p.ld + j];
            long long xr = __double2ll_rn(ldexp(a.x, GBPERM_FIX_BITS - e));
            long long xi = __double2ll_rn(ldexp(a.y, GBPERM_FIX_BITS - e));
            p.a1[i * p.cols + j] = make_longlong2(xr, xi);
            p.a2[i * p.cols + j] = make_longlong2(2 * xr, 2 * xi);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long tot = 0;
        for (int j = 0; j < p.cols; ++j) tot += (long long)s_e[j] * (p.col_w ? p.col_w[j] : 1);
        p.exp_out[0] = (int)(tot - p.norm_shift);
    }
}

}  // namespace

cudaError_t launch_prepare(const PrepArgs& a, cudaStream_t st) {
    prepare_kernel<<<1, 64, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace gbperm
