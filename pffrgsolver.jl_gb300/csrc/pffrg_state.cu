// Elementwise action kernels (sm_103a), FP64: the v <-> v' symmetrisation of
// the vertex (src/Action/action_lib/action_su2.jl:141-251), the Bogacki-Shampine
// stage algebra (src/Action/Action.jl:181-337 as used by
// src/Launcher/launcher_{1l,2l,ml}.jl) and the error norm get_abs_max
// (Action.jl:346-359, channel.jl:406-413: maximum |q3|).  All are HBM
// streaming kernels with grid-stride loops over the packed layout.
#include "pffrg_internal.h"

namespace pffrg {

static int grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    const int64_t cap = 152 * 16;
    return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

// image of (component c, channel ch) under v <-> v': the component it is read
// from and the sign (SU(2): itself, +; U(1)-DM, action_u1_dm.jl:170-339: s and t
// channels DM -> -DM, zd -> -dz, dz -> -zd; u channel zd -> -zd, dz -> -dz)
__device__ __forceinline__ int swap_image(int C, int c, int ch, double& sgn) {
    sgn = 1.0;
    if (C == 2) return c;
    if (ch == 2) {
        if (c == 4 || c == 5) sgn = -1.0;
        return c;
    }
    if (c == 2) sgn = -1.0;
    if (c == 4 || c == 5) {
        sgn = -1.0;
        return 9 - c;
    }
    return c;
}

// symmetrize!: q3[i,w,v,v'] = ± q3'[x(i),w,v',v] for v < v', x = exchange (s, t) or identity (u)
__global__ void symmetrize_kernel(Layout L, const int* __restrict__ exch, double* a) {
    const int Ns = L.Ns, NO = L.NO, Nn = L.Nn;
    const int64_t npair = (int64_t)Nn * (Nn - 1) / 2;
    const int64_t per = npair * NO * Ns;
    const int64_t n = per * 3 * L.C;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = e;
        const int i = (int)(r % Ns);
        r /= Ns;
        const int w = (int)(r % NO);
        r /= NO;
        int64_t pr = r % npair;
        r /= npair;
        const int ch = (int)(r % 3);
        const int c = (int)(r / 3);
        // pair index -> (v < vp)
        int v = 0;
        while (pr >= Nn - 1 - v) {
            pr -= Nn - 1 - v;
            ++v;
        }
        const int vp = v + 1 + (int)pr;
        double sgn;
        const int sc = swap_image(L.C, c, ch, sgn);
        double* q3 = a + L.qbase(c, ch, 3);
        const double* s3 = a + L.qbase(sc, ch, 3);
        const int src = ch == 2 ? i : exch[i];
        // the lower triangle read here is never written
        q3[i + (int64_t)Ns * (w + (int64_t)NO * (v + (int64_t)Nn * vp))] =
            sgn * s3[src + (int64_t)Ns * (w + (int64_t)NO * (vp + (int64_t)Nn * v))];
    }
}

// symmetrize_add_to!: a += a_l + (v <-> v') image of a_l, on q1, q2_1/q2_2 and q3
__global__ void symmetrize_add_kernel(Layout L, const int* __restrict__ exch, const double* __restrict__ al,
                                      double* a) {
    const int Ns = L.Ns, NO = L.NO, Nn = L.Nn;
    const int64_t n = L.chan * 3 * L.C;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = e % L.chan;
        const int64_t cc = e / L.chan;
        const int ch = (int)(cc % 3), c = (int)(cc / 3);
        const int64_t base = L.qbase(c, ch, 0);
        double sgn;
        const int64_t sbase = L.qbase(swap_image(L.C, c, ch, sgn), ch, 0);
        const int i = (int)(k % Ns);
        const int ex = ch == 2 ? i : exch[i];
        int64_t src;
        if (k < L.K1) {
            src = sbase + (k - i + ex);
        } else if (k < L.K1 + 2 * L.K2) {
            const bool first = k < L.K1 + L.K2;
            const int64_t kk = first ? k - L.K1 : k - L.K1 - L.K2;
            // q2_1 <- q2_2 image and q2_2 <- q2_1 image at the exchanged site
            src = sbase + (first ? L.K1 + L.K2 : L.K1) + (kk - i + ex);
        } else {
            const int64_t kk = k - L.K1 - 2 * L.K2;
            int64_t r = kk / Ns;
            const int w = (int)(r % NO);
            r /= NO;
            const int v = (int)(r % Nn);
            const int vp = (int)(r / Nn);
            src = sbase + L.K1 + 2 * L.K2 + ex + (int64_t)Ns * (w + (int64_t)NO * (vp + (int64_t)Nn * v));
        }
        a[base + k] += al[base + k] + sgn * al[src];
    }
}

// y = alpha * y + beta * x on Σ (optional) and the channels (bare excluded)
__global__ void axpby_kernel(Layout L, double alpha, const double* __restrict__ x, double beta, double* y,
                             bool sigma_too, bool gamma_too) {
    const int64_t ng = gamma_too ? L.C * 3 * L.chan : 0;
    const int64_t ns = sigma_too ? L.Nsig : 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ns + ng; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t idx;
        if (e < ns) {
            idx = e;
        } else {
            const int64_t g = e - ns;
            const int c = (int)(g / (3 * L.chan));
            idx = L.qbase(c, 0, 0) + g % (3 * L.chan);
        }
        const double xv = x ? beta * x[idx] : 0.0;
        y[idx] = (alpha == 0.0 ? 0.0 : alpha * y[idx]) + xv;
    }
}

__global__ void to_float_kernel(const double* __restrict__ x, float* y, int64_t n) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        y[e] = (float)x[e];
}

__global__ void absmax_partial_kernel(Layout L, const double* __restrict__ a, double* partial) {
    const int64_t per = L.K3;
    const int64_t n = per * 3 * L.C;
    double m = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t cc = e / per;
        const int ch = (int)(cc % 3), c = (int)(cc / 3);
        m = fmax(m, fabs(a[L.qbase(c, ch, 3) + e % per]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < blockDim.x / 32 ? sm[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

__global__ void max_reduce_kernel(const double* partial, int n, double* out) {
    double m = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) m = fmax(m, partial[k]);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ double sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < blockDim.x / 32 ? sm[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) out[0] = v;
    }
}

cudaError_t launch_symmetrize(const Layout& L, const int* exch, double* a, cudaStream_t st) {
    const int64_t n = (int64_t)L.Nn * (L.Nn - 1) / 2 * L.NO * L.Ns * 3 * L.C;
    if (n == 0) return cudaSuccess;
    symmetrize_kernel<<<grid_for(n, 256), 256, 0, st>>>(L, exch, a);
    return cudaGetLastError();
}

cudaError_t launch_symmetrize_add_to(const Layout& L, const int* exch, const double* al, double* a,
                                     cudaStream_t st) {
    const int64_t n = L.chan * 3 * L.C;
    symmetrize_add_kernel<<<grid_for(n, 256), 256, 0, st>>>(L, exch, al, a);
    return cudaGetLastError();
}

cudaError_t launch_axpby(const Layout& L, double alpha, const double* x, double beta, double* y, bool sigma_too,
                         bool gamma_too, cudaStream_t st) {
    const int64_t n = (sigma_too ? L.Nsig : 0) + (gamma_too ? L.C * 3 * L.chan : 0);
    axpby_kernel<<<grid_for(n, 256), 256, 0, st>>>(L, alpha, x, beta, y, sigma_too, gamma_too);
    return cudaGetLastError();
}

cudaError_t launch_to_float(const double* x, float* y, int64_t n, cudaStream_t st) {
    to_float_kernel<<<grid_for(n, 256), 256, 0, st>>>(x, y, n);
    return cudaGetLastError();
}

cudaError_t launch_absmax_q3(const Layout& L, const double* a, double* partial, int npartial, double* out,
                             cudaStream_t st) {
    absmax_partial_kernel<<<npartial, 256, 0, st>>>(L, a, partial);
    max_reduce_kernel<<<1, 256, 0, st>>>(partial, npartial, out);
    return cudaGetLastError();
}

}  // namespace pffrg
