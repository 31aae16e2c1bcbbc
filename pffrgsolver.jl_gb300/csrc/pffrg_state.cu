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

// status bit 4 (16) when any of the n values is NaN or infinite: a right-hand side whose result is
// not finite is reported as PFFRG_E_NONFINITE instead of flowing into the next ODE stage
__global__ void finite_kernel(const double* __restrict__ a, int64_t n, int* status) {
    int bad = 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        bad |= !isfinite(a[e]);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(status, 16);
}

// the SDE iteration's errors (parquet.jl:59-61): out = [max|ap.Σ - a.Σ|, max|a.Σ|, max|ap.Σ|]
__global__ void sigma_err_kernel(int Nsig, const double* __restrict__ a, const double* __restrict__ ap, double* out) {
    double d = 0.0, ma = 0.0, mp = 0.0;
    for (int k = threadIdx.x; k < Nsig; k += blockDim.x) {
        d = fmax(d, fabs(ap[k] - a[k]));
        ma = fmax(ma, fabs(a[k]));
        mp = fmax(mp, fabs(ap[k]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        d = fmax(d, __shfl_xor_sync(0xffffffffu, d, o));
        ma = fmax(ma, __shfl_xor_sync(0xffffffffu, ma, o));
        mp = fmax(mp, __shfl_xor_sync(0xffffffffu, mp, o));
    }
    if (threadIdx.x == 0) {
        out[0] = d;
        out[1] = ma;
        out[2] = mp;
    }
}

// FP32 copy of an SU(2) action with the two components of every entry side by side (Layout::pq):
// Σ as is, then (spin, density) pairs of bare and every channel array
__global__ void to_float_pairs_kernel(Layout L, const double* __restrict__ x, float* y) {
    const int64_t np = L.comp;  // entries per component after Σ
    float2* y2 = reinterpret_cast<float2*>(y) + L.pbare();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < np + L.Nsig;
         e += (int64_t)gridDim.x * blockDim.x) {
        if (e < np) y2[e] = make_float2((float)x[L.Nsig + e], (float)x[L.Nsig + L.comp + e]);
        else y[e - np] = (float)x[e - np];
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

// ---------------------------------------------------------------------------
// mesh scanning and resampling between flow steps (Action.jl:361-557, channel.jl:416-471)
// ---------------------------------------------------------------------------
// argmax |q3| of every (component, channel), the first of equal maxima in column-major order
// (Julia's argmax), and the four cuts through it that scan_channel reads (Action.jl:452-480):
// q3[s, :, v, v'], q3[s, w, k, k] - q3[s, w, end, end], q3[s, w, :, v'] - q3[s, w, end, v'],
// q3[s, w, v, :] - q3[s, w, v, end].  One block per (component, channel).
__global__ void scan_cuts_kernel(Layout L, const double* __restrict__ a, long long* argmax, double* cuts) {
    const int cc = blockIdx.x;  // component * 3 + channel
    const int c = cc / 3, ch = cc % 3;
    const double* q3 = a + L.qbase(c, ch, 3);
    double best = -1.0;
    long long bi = 0;
    for (long long e = threadIdx.x; e < L.K3; e += blockDim.x) {
        const double m = fabs(q3[e]);
        if (m > best) {  // the first maximum of this thread's stride
            best = m;
            bi = e;
        }
    }
    __shared__ double sb[32];
    __shared__ long long si[32];
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    if ((threadIdx.x & 31) == 0) {
        sb[threadIdx.x >> 5] = best;
        si[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x / 32;
        best = threadIdx.x < nw ? sb[threadIdx.x] : -1.0;
        bi = threadIdx.x < nw ? si[threadIdx.x] : 0x7fffffffffffffffll;
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (threadIdx.x == 0) si[0] = bi;
    }
    __syncthreads();
    bi = si[0];
    const int Ns = L.Ns, NO = L.NO, Nn = L.Nn;
    long long r = bi;
    const int s = (int)(r % Ns);
    r /= Ns;
    const int w = (int)(r % NO);
    r /= NO;
    const int v = (int)(r % Nn);
    const int vp = (int)(r / Nn);
    auto at = [&](int ww, int x, int y) { return q3[s + (long long)Ns * (ww + (long long)NO * (x + (long long)Nn * y))]; };
    double* out = cuts + (size_t)cc * (NO + 3 * Nn);
    for (int k = threadIdx.x; k < NO; k += blockDim.x) out[k] = at(k, v, vp);
    for (int k = threadIdx.x; k < Nn; k += blockDim.x) {
        out[NO + k] = at(w, k, k) - at(w, Nn - 1, Nn - 1);
        out[NO + Nn + k] = at(w, k, vp) - at(w, Nn - 1, vp);
        out[NO + 2 * Nn + k] = at(w, v, k) - at(w, v, Nn - 1);
    }
    if (threadIdx.x == 0) argmax[cc] = bi;
}

// resample_from_to (Action.jl:537-557): Σ by get_Σ on the old σ mesh, every q by the multilinear
// interpolation of the old channel at the new frequencies (channel.jl:416-471), bare copied.
// mesh_old / mesh_new: [σ | Ωs | νs | Ωt | νt] blocks.
__global__ void resample_kernel(Layout L, const double* __restrict__ mesh_old, const double* __restrict__ mesh_new,
                                const double* __restrict__ a, double* b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SMesh<double>& M = *reinterpret_cast<SMesh<double>*>(smem_raw);
    load_mesh(M, mesh_old, L.Nsig, L.NO, L.Nn);
    __syncthreads();
    const int Ns = L.Ns, NO = L.NO, Nn = L.Nn;
    const double* sig_new = mesh_new;
    const double* Os_new = sig_new + L.Nsig;
    const double* ns_new = Os_new + NO;
    const double* Ot_new = ns_new + Nn;
    const double* nt_new = Ot_new + NO;
    const long long n = L.total;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        if (e < L.Nsig) {
            b[e] = get_sigma(M, L.Nsig, a, sig_new[e]);
            continue;
        }
        const long long in_comp = (e - L.Nsig) % L.comp;
        if (in_comp < Ns) {  // bare
            b[e] = a[e];
            continue;
        }
        const long long rc = in_comp - Ns;
        const int ch = (int)(rc / L.chan);
        long long k = rc % L.chan;
        const double* Om = ch == 1 ? M.Ot : M.Os;
        const double* iOm = ch == 1 ? M.iOt : M.iOs;
        const double* nu = ch == 1 ? M.nt : M.ns;
        const double* inu = ch == 1 ? M.int_ : M.ins;
        const double* Onew = ch == 1 ? Ot_new : Os_new;
        const double* nnew = ch == 1 ? nt_new : ns_new;
        const double* q = a + (e - in_comp) + Ns + (long long)ch * L.chan;  // this channel of the old action
        const int s = (int)(k % Ns);
        double val;
        if (k < L.K1) {  // q1 (channel.jl:55-75)
            const int w = (int)(k / Ns);
            const Param<double> p1 = get_param(Onew[w], Om, iOm, NO);
            val = p1.wl * q[s + (long long)Ns * p1.lo];
            val += p1.wu * q[s + (long long)Ns * p1.hi];
        } else if (k < L.K1 + 2 * L.K2) {  // q2_1, q2_2 (channel.jl:104-184)
            const bool first = k < L.K1 + L.K2;
            const long long kk = k - L.K1 - (first ? 0 : L.K2);
            const int w = (int)((kk / Ns) % NO), v = (int)(kk / ((long long)Ns * NO));
            const Param<double> pa = get_param(Onew[w], Om, iOm, NO);
            const Param<double> pb = get_param(nnew[v], nu, inu, Nn);
            const double* Q = q + L.K1 + (first ? 0 : L.K2);
            auto ix = [&](int ww, int vv) { return s + (long long)Ns * (ww + (long long)NO * vv); };
            val = pa.wl * pb.wl * Q[ix(pa.lo, pb.lo)];
            val += pa.wu * pb.wl * Q[ix(pa.hi, pb.lo)];
            val += pa.wl * pb.wu * Q[ix(pa.lo, pb.hi)];
            val += pa.wu * pb.wu * Q[ix(pa.hi, pb.hi)];
        } else {  // q3 (channel.jl:226-305)
            const long long kk = k - L.K1 - 2 * L.K2;
            long long r = kk / Ns;
            const int w = (int)(r % NO);
            r /= NO;
            const int v = (int)(r % Nn), vp = (int)(r / Nn);
            const Param<double> p1 = get_param(Onew[w], Om, iOm, NO);
            const Param<double> p2 = get_param(nnew[v], nu, inu, Nn);
            const Param<double> p3 = get_param(nnew[vp], nu, inu, Nn);
            const double* Q = q + L.K1 + 2 * L.K2;
            auto ix = [&](int ww, int x, int y) {
                return s + (long long)Ns * (ww + (long long)NO * (x + (long long)Nn * y));
            };
            val = p1.wl * p2.wl * p3.wl * Q[ix(p1.lo, p2.lo, p3.lo)];
            val += p1.wu * p2.wl * p3.wl * Q[ix(p1.hi, p2.lo, p3.lo)];
            val += p1.wl * p2.wu * p3.wl * Q[ix(p1.lo, p2.hi, p3.lo)];
            val += p1.wu * p2.wu * p3.wl * Q[ix(p1.hi, p2.hi, p3.lo)];
            val += p1.wl * p2.wl * p3.wu * Q[ix(p1.lo, p2.lo, p3.hi)];
            val += p1.wu * p2.wl * p3.wu * Q[ix(p1.hi, p2.lo, p3.hi)];
            val += p1.wl * p2.wu * p3.wu * Q[ix(p1.lo, p2.hi, p3.hi)];
            val += p1.wu * p2.wu * p3.wu * Q[ix(p1.hi, p2.hi, p3.hi)];
        }
        b[e] = val;
    }
}

cudaError_t launch_scan_cuts(const Layout& L, const double* a, long long* argmax, double* cuts, cudaStream_t st) {
    scan_cuts_kernel<<<3 * L.C, 256, 0, st>>>(L, a, argmax, cuts);
    return cudaGetLastError();
}

cudaError_t launch_resample(const Layout& L, const double* mesh_old, const double* mesh_new, const double* a,
                            double* b, cudaStream_t st) {
    const size_t smem = sizeof(SMesh<double>);
    cudaError_t e = cudaFuncSetAttribute(resample_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    resample_kernel<<<grid_for(L.total, 256), 256, smem, st>>>(L, mesh_old, mesh_new, a, b);
    return cudaGetLastError();
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

cudaError_t launch_sigma_err(int Nsig, const double* a, const double* ap, double* out, cudaStream_t st) {
    sigma_err_kernel<<<1, 32, 0, st>>>(Nsig, a, ap, out);
    return cudaGetLastError();
}

cudaError_t launch_check_finite(const double* a, int64_t n, int* status, cudaStream_t st) {
    finite_kernel<<<grid_for(n, 256), 256, 0, st>>>(a, n, status);
    return cudaGetLastError();
}

cudaError_t launch_to_float_pairs(const Layout& L, const double* x, float* y, cudaStream_t st) {
    to_float_pairs_kernel<<<grid_for(L.comp + L.Nsig, 256), 256, 0, st>>>(L, x, y);
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
