// Fixed-point preparation of one matrix on the device (see gbperm_internal.h).
#include <cmath>
#include <vector>

#include "gbperm_internal.h"

namespace gbperm {

namespace {

__global__ void prepare_kernel(PrepArgs p) {
    const int bt = blockIdx.x;  // matrix of a batch
    if (bt > 0) {
        p.A += (long long)bt * p.a_stride;
        p.a1 += (size_t)bt * p.rows * p.cols;
        p.a2 += (size_t)bt * p.rows * p.cols;
        p.exp_out += bt;
        if (p.exp_fp64_out) p.exp_fp64_out += bt;
        if (p.row_k_out) p.row_k_out += (size_t)bt * p.rows;
        if (p.col_e_out) p.col_e_out += (size_t)bt * p.cols;
        if (p.df_info) p.df_info += 2 * bt;
    }
    __shared__ int s_e[64];
    __shared__ double s_typ[64];
    __shared__ int s_k[64];  // row scaling exponents
    for (int i = threadIdx.x; i < p.rows; i += blockDim.x) {
        int k = 0;
        if (p.row_balance) {
            double mx = 0.0;
            for (int j = 0; j < p.cols; ++j) {
                const double2 a = p.A[(long long)i * p.ld + j];
                mx = fmax(mx, fmax(fabs(a.x), fabs(a.y)));
            }
            if (mx > 0.0) frexp(mx, &k);
        }
        s_k[i] = k;
        if (p.row_k_out) p.row_k_out[i] = k;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < p.cols; j += blockDim.x) {
        double br = 0.0, bi = 0.0, l2 = 0.0;
        for (int i = 0; i < p.rows; ++i) {
            double2 a = p.A[(long long)i * p.ld + j];
            a.x = ldexp(a.x, -s_k[i]);
            a.y = ldexp(a.y, -s_k[i]);
            double w = p.row_w ? (double)p.row_w[i] : 1.0;
            br += w * fabs(a.x);
            bi += w * fabs(a.y);
            if (p.df) l2 += w * (a.x * a.x + a.y * a.y);
        }
        // a little headroom so that rounding in the bound never lets a sum
        // reach 2^62 in fixed point
        double b = fmax(br, bi) * (1.0 + 1e-12);
        int e = 0;
        if (b > 0.0) frexp(b, &e);
        s_e[j] = e;
        if (p.col_e_out) p.col_e_out[j] = e;
        // the typical column size only feeds the double-float range boost
        // (the FP64 pipe is slow on GB300: skip the log2 otherwise)
        s_typ[j] = (p.df && b > 0.0) ? log2(sqrt(l2) / ldexp(1.0, e)) : -1e300;
        for (int i = 0; i < p.rows; ++i) {
            double2 a = p.A[(long long)i * p.ld + j];
            long long xr = __double2ll_rn(ldexp(a.x, GBPERM_FIX_BITS - e - s_k[i]));
            long long xi = __double2ll_rn(ldexp(a.y, GBPERM_FIX_BITS - e - s_k[i]));
            p.a1[i * p.cols + j] = make_longlong2(xr, xi);
            p.a2[i * p.cols + j] = make_longlong2(2 * xr, 2 * xi);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long tot = 0;
        long long pw = 0;
        double typ = 0.0;
        for (int j = 0; j < p.cols; ++j) {
            long long w = p.col_w ? p.col_w[j] : 1;
            tot += (long long)s_e[j] * w;
            pw += w;
            if (w) typ += (double)w * s_typ[j];
        }
        for (int i = 0; i < p.rows; ++i) tot += (long long)s_k[i] * (p.row_w ? p.row_w[i] : 1);
        if (p.exp_fp64_out) p.exp_fp64_out[0] = (int)(tot - p.norm_shift);
        if (p.df) {
            // range boost o of the double-float product: centre the typical
            // term near 2^-40, keep the largest possible one below 2^118
            int o = 0, ok = 0;
            if (pw > 0 && typ > -1e290) {
                o = (int)floor((-40.0 - typ) / (double)pw);
                int omax = (int)floor(118.0 / (double)pw - 0.5);
                if (o > omax) o = omax;
                ok = (typ + (double)o * (double)pw >= -100.0) ? 1 : 0;
            }
            if (!ok) o = 0;
            tot -= (long long)o * pw;
            p.df_info[0] = o;
            p.df_info[1] = ok;
        }
        p.exp_out[0] = (int)(tot - p.norm_shift);
    }
}

}  // namespace

bool df_boost(const double* A, int64_t rows, int64_t cols, int64_t ld, const int* row_w,
              const int* col_w, int* boost, bool row_balance) {
    double typ = 0.0;   // log2 of the typical |term| before the boost
    double pw = 0.0;    // number of factors
    std::vector<int> k(rows > 0 ? rows : 1, 0);  // the prepare kernel's row exponents
    if (row_balance)
        for (int64_t i = 0; i < rows; ++i) {
            double mx = 0.0;
            for (int64_t j = 0; j < cols; ++j)
                mx = std::fmax(mx, std::fmax(std::fabs(A[2 * (i * ld + j)]), std::fabs(A[2 * (i * ld + j) + 1])));
            if (mx > 0.0) std::frexp(mx, &k[i]);
        }
    for (int64_t j = 0; j < cols; ++j) {
        double br = 0.0, bi = 0.0, l2 = 0.0;
        for (int64_t i = 0; i < rows; ++i) {
            double w = row_w ? (double)row_w[i] : 1.0;
            double re = std::ldexp(A[2 * (i * ld + j)], -k[i]), im = std::ldexp(A[2 * (i * ld + j) + 1], -k[i]);
            br += w * std::fabs(re);
            bi += w * std::fabs(im);
            l2 += w * (re * re + im * im);
        }
        double b = std::fmax(br, bi) * (1.0 + 1e-12);
        double w = col_w ? (double)col_w[j] : 1.0;
        if (w == 0.0) continue;
        if (b == 0.0) return false;  // a zero column: permanent 0, no range issue but no scale either
        int e = 0;
        std::frexp(b, &e);
        typ += w * std::log2(std::sqrt(l2) / std::ldexp(1.0, e));
        pw += w;
    }
    if (pw == 0.0) return false;
    int o = (int)std::floor((-40.0 - typ) / pw);
    int omax = (int)std::floor(118.0 / pw - 0.5);
    if (o > omax) o = omax;
    if (typ + o * pw < -100.0) return false;
    *boost = o;
    return true;
}

cudaError_t launch_prepare(const PrepArgs& a, cudaStream_t st) {
    prepare_kernel<<<a.count, 64, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace gbperm
