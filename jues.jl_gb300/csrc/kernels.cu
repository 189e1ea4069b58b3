// Bandwidth-bound kernels: permutations, energies, amplitude finalisation, DIIS vectors.
//
// Every reduction is deterministic: a fixed-size grid writes one FP64 partial per block,
// and a single block sums the partials in a fixed order.
#include <algorithm>
#include <atomic>
#include <cmath>

#include "common.cuh"

namespace jues {

namespace {

constexpr int RED_BLOCKS = 1184;   // 8 blocks per SM on 148-152 SM parts; fixed for determinism
constexpr int RED_THREADS = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// up to 16 vectors and coefficients as one kernel argument
struct VecList {
    const double *p[16];
    double c[16];
};

// warp-wide sum, valid in every lane
__device__ __forceinline__ double warp_allsum(double v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// block-wide sum; result valid in thread 0
__device__ __forceinline__ double block_sum(double v) {
    __shared__ double s[32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) s[w] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? s[threadIdx.x] : 0.0;
    if (w == 0) v = warp_sum(v);
    return v;
}

__global__ void reduce_partials(const double *part, int n, double *out) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
    v = block_sum(v);
    if (threadIdx.x == 0) *out = v;
}

__global__ void permute4_kernel(Perm4 p, double alpha, const double *__restrict__ in, double beta,
                                double *__restrict__ out, long long total) {
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < total;
         x += (long long)gridDim.x * blockDim.x) {
        long long r = x;
        long long i0 = r % p.d[0]; r /= p.d[0];
        long long i1 = r % p.d[1]; r /= p.d[1];
        long long i2 = r % p.d[2]; long long i3 = r / p.d[2];
        long long oi = i0 * p.si[0] + i1 * p.si[1] + i2 * p.si[2] + i3 * p.si[3];
        long long oo = i0 * p.so[0] + i1 * p.so[1] + i2 * p.so[2] + i3 * p.so[3];
        double v = alpha * in[oi];
        if (beta != 0.0) v += beta * out[oo];
        out[oo] = v;
    }
}

// Tiled form of permute4_kernel for a permutation that moves the input's unit-stride dimension
// (ki) away from the output's (ko): a 32 x 32 tile of the (ki, ko) plane goes through shared
// memory, so both the loads (along ki) and the stores (along ko) are coalesced.  VEC: 16-byte
// loads and stores (two doubles per thread; the host checks alignment and even extents).
// Block 32 x 8 threads; grid x = tiles of the plane, grid y strides over the other two dimensions.
template <bool VEC>
__global__ void __launch_bounds__(256) permute4_tiled_kernel(Perm4 p, int ki, int ko, int r1, int r2, double alpha,
                                                             const double *__restrict__ in, double beta,
                                                             double *__restrict__ out) {
    __shared__ double tile[32][33];   // [ko][ki], odd pitch: column reads are conflict-free
    const long long dki = p.d[ki], dko = p.d[ko];
    const long long nti = (dki + 31) / 32;
    const long long ti = blockIdx.x % nti, to = blockIdx.x / nti;
    const long long i0 = ti * 32, o0 = to * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long long nrest = p.d[r1] * p.d[r2];
    for (long long rest = blockIdx.y; rest < nrest; rest += gridDim.y) {
        const long long a1 = rest % p.d[r1], a2 = rest / p.d[r1];
        const long long bin = a1 * p.si[r1] + a2 * p.si[r2], bout = a1 * p.so[r1] + a2 * p.so[r2];
        if (VEC) {
            // lanes 0-15 load row y, lanes 16-31 row y + 1, two consecutive ki each
            const int c = 2 * (tx & 15), rsub = tx >> 4;
            for (int y = 2 * ty + rsub; y < 32; y += 16) {
                const long long k = i0 + c, q = o0 + y;
                if (q < dko && k < dki) {
                    const double2 v = *reinterpret_cast<const double2 *>(in + bin + k + q * p.si[ko]);
                    tile[y][c] = v.x;
                    tile[y][c + 1] = v.y;
                }
            }
            __syncthreads();
            for (int y = 2 * ty + rsub; y < 32; y += 16) {
                const long long q = o0 + c, k = i0 + y;
                if (k < dki && q < dko) {
                    double2 *dst = reinterpret_cast<double2 *>(out + bout + q + k * p.so[ki]);
                    double2 v = make_double2(alpha * tile[c][y], alpha * tile[c + 1][y]);
                    if (beta != 0.0) {
                        const double2 w = *dst;
                        v.x = fma(beta, w.x, v.x);
                        v.y = fma(beta, w.y, v.y);
                    }
                    *dst = v;
                }
            }
        } else {
            for (int y = ty; y < 32; y += 8) {
                const long long k = i0 + tx, q = o0 + y;
                if (q < dko && k < dki) tile[y][tx] = in[bin + k + q * p.si[ko]];
            }
            __syncthreads();
            for (int y = ty; y < 32; y += 8) {
                const long long q = o0 + tx, k = i0 + y;
                if (k < dki && q < dko) {
                    double *dst = out + bout + q + k * p.so[ki];
                    double v = alpha * tile[tx][y];
                    if (beta != 0.0) v = fma(beta, *dst, v);
                    *dst = v;
                }
            }
        }
        __syncthreads();
    }
}

__global__ void fill_kernel(double *p, size_t n, double v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void axpby_kernel(size_t n, double a, const double *__restrict__ x, double b,
                             const double *__restrict__ y, double *__restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = a * x[i] + (y ? b * y[i] : 0.0);
}

__global__ void dot_kernel(size_t n, const double *__restrict__ x, const double *__restrict__ y,
                           double *part) {
    double v = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        v = fma(x[i], y[i], v);
    v = block_sum(v);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
}

__global__ void nonfinite_kernel(size_t n, const double *__restrict__ x, unsigned *flag) {
    bool bad = false;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        bad |= !isfinite(x[i]);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1u);
}

// pair index p (a <= b) -> (a, b)
__device__ __forceinline__ void pair_ab(long long p, int &a, int &b) {
    long long bb = (long long)((sqrt(8.0 * (double)p + 1.0) - 1.0) * 0.5);
    while (bb * (bb + 1) / 2 > p) --bb;
    while ((bb + 1) * (bb + 2) / 2 <= p) ++bb;
    b = (int)bb;
    a = (int)(p - bb * (bb + 1) / 2);
}

// the same for p < 2^26 in FP32 and 32-bit integers (the FP64 square root is slow on this part)
__device__ __forceinline__ void pair_ab32(int p, int &a, int &b) {
    int bb = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
    while (bb * (bb + 1) / 2 > p) --bb;
    while ((bb + 1) * (bb + 2) / 2 <= p) ++bb;
    b = bb;
    a = p - bb * (bb + 1) / 2;
}

// MP2: each (a<=b) pair block reads K[:,:,a,b] and K[:,:,b,a] once.
__global__ void mp2_kernel(const double *__restrict__ K, const double *__restrict__ eps, int o, int v,
                           double *part) {
    const long long oo = (long long)o * o;
    const long long npair = (long long)v * (v + 1) / 2;
    double acc = 0.0;
    for (long long p = blockIdx.x; p < npair; p += gridDim.x) {
        int a, b;
        pair_ab(p, a, b);
        const double ea = eps[o + a], eb = eps[o + b];
        const double *Kab = K + oo * (a + (long long)v * b);
        const double *Kba = K + oo * (b + (long long)v * a);
        for (long long ij = threadIdx.x; ij < oo; ij += blockDim.x) {
            int i = (int)(ij % o), j = (int)(ij / o);
            double inv = 1.0 / (eps[i] + eps[j] - ea - eb);
            double x = Kab[ij];
            if (a == b) {
                acc = fma(x * x, inv, acc);
            } else {
                double y = Kba[ij];
                acc = fma(x * (2.0 * x - y) + y * (2.0 * y - x), inv, acc);
            }
        }
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// CC energy: sum oovv[i,j,a,b] (2X[i,j,a,b] - X[j,i,a,b]), X = T2 + t1(x)t1
__global__ void ccenergy_kernel(const double *__restrict__ W, const double *__restrict__ T,
                                const double *__restrict__ t1, int o, int v, double *part) {
    const long long oo = (long long)o * o, vv = (long long)v * v;
    double acc = 0.0;
    for (long long ab = blockIdx.x; ab < vv; ab += gridDim.x) {
        const int a = (int)(ab % v), b = (int)(ab / v);
        const double *Wb = W + oo * ab;
        const double *Tb = T + oo * ab;
        for (long long ij = threadIdx.x; ij < oo; ij += blockDim.x) {
            int i = (int)(ij % o), j = (int)(ij / o);
            double x = Tb[ij], y = Tb[j + (long long)o * i];
            if (t1) {
                x += t1[i + (long long)o * a] * t1[j + (long long)o * b];
                y += t1[j + (long long)o * a] * t1[i + (long long)o * b];
            }
            acc = fma(Wb[ij], 2.0 * x - y, acc);
        }
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// 1 / D[i,j,a,b] = 1 / (e_i + e_j - e_a - e_b), formed once per CC problem: GB300 runs FP64 at a
// few operations per clock per SM, so an FP64 division per element would dominate the sweep's
// finalisation; the sweeps then multiply.
__global__ void inv_denominators_kernel(const double *__restrict__ eps, int o, int v, double *__restrict__ out) {
    const long long oo = (long long)o * o, n = oo * v * v;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
         x += (long long)gridDim.x * blockDim.x) {
        long long ij = x % oo, ab = x / oo;
        int i = (int)(ij % o), j = (int)(ij / o), a = (int)(ab % v), b = (int)(ab / v);
        out[x] = 1.0 / (eps[i] + eps[j] - eps[o + a] - eps[o + b]);
    }
}

// the same over the pairs: out[p + np q] = 1/D[i0,j0,a,b] for p = (i0 <= j0), q = (a <= b), with
// the sums in inv_denominators_kernel's order (so equal to its entry at (i0,j0,a,b) to the bit)
__global__ void inv_denominators_folded_kernel(const double *__restrict__ eps, int o, int v, double *__restrict__ out) {
    const int np = o * (o + 1) / 2;
    const long long n = (long long)np * v * (v + 1) / 2;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
         x += (long long)gridDim.x * blockDim.x) {
        int i, j, a, b;
        pair_ab32((int)(x % np), i, j);
        pair_ab32((int)(x / np), a, b);
        out[x] = 1.0 / (eps[i] + eps[j] - eps[o + a] - eps[o + b]);
    }
}

// Tn[i,j,a,b] = (L[i,j,a,b] + Z[i,j,a,b] + Z[j,i,b,a] + C[i,j,a,b] + C[j,i,b,a]) / D with the
// optional rank-one C[i,j,a,b] = t1[i,a] q[b,j] (t1 o x v, q v x o), and the squared step norm.
__device__ __forceinline__ double rank1_pair(const double *__restrict__ t1, const double *__restrict__ q, int o,
                                             int v, int i, int j, int a, int b) {
    return t1[i + (long long)o * a] * q[b + (long long)v * j] + t1[j + (long long)o * b] * q[a + (long long)v * i];
}
__global__ void t2_finalize_kernel(const double *__restrict__ L, const double *__restrict__ Z,
                                   const double *__restrict__ invD, int o, int v,
                                   const double *__restrict__ Told, double *__restrict__ Tn,
                                   double *part, const double *__restrict__ t1, const double *__restrict__ q) {
    const long long oo = (long long)o * o;
    const long long npair = (long long)v * (v + 1) / 2;
    double acc = 0.0;
    for (long long p = blockIdx.x; p < npair; p += gridDim.x) {
        int a, b;
        pair_ab(p, a, b);
        const long long ab = oo * (a + (long long)v * b), ba = oo * (b + (long long)v * a);
        for (long long ij = threadIdx.x; ij < oo; ij += blockDim.x) {
            int i = (int)(ij % o), j = (int)(ij / o);
            long long ji = j + (long long)o * i;
            const double inv = invD[ab + ij];   // D is symmetric in (a, b)
            double x = L[ab + ij] + Z[ab + ij] + Z[ba + ji];
            if (t1) x += rank1_pair(t1, q, o, v, i, j, a, b);
            x *= inv;
            Tn[ab + ij] = x;
            if (Told) { double d = x - Told[ab + ij]; acc = fma(d, d, acc); }
            if (a != b) {
                double y = L[ba + ij] + Z[ba + ij] + Z[ab + ji];
                if (t1) y += rank1_pair(t1, q, o, v, i, j, b, a);
                y *= inv;
                Tn[ba + ij] = y;
                if (Told) { double d = y - Told[ba + ij]; acc = fma(d, d, acc); }
            }
        }
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// The same finalisation with the (i,j) transposes through shared memory: block p handles the
// pair (a <= b) (one pair per block, so resident blocks overlap their load and compute phases);
// Z[:,:,a,b] and Z[:,:,b,a] are contiguous o x o blocks, loaded coalesced into shared memory on
// an odd row pitch (conflict-free transposed reads), so every global access is unit-stride.
// Dynamic shared memory 2 o pitch doubles (o <= 64), + 4 o with the rank-one term.
template <bool RANK1>
__global__ void __launch_bounds__(256, RANK1 ? 6 : 8) t2_finalize_smem_kernel(const double *__restrict__ L,
                                                               const double *__restrict__ Z,
                                                               const double *__restrict__ invD, int o, int v,
                                                               const double *__restrict__ Told,
                                                               double *__restrict__ Tn, double *part,
                                                               const double *__restrict__ t1,
                                                               const double *__restrict__ q) {
    extern __shared__ double zs[];   // [2][o][pitch]: zs[0] = Z_ab, zs[1] = Z_ba, element (i, j) at j + pitch i
    // RANK1: then t1[:,a], t1[:,b], q[a,:], q[b,:] (o each)
    const int pitch = o | 1;
    const long long oo = (long long)o * o;
    const int ooi = o * o;
    double acc = 0.0;
    int a, b;
    pair_ab32((int)blockIdx.x, a, b);   // one (a <= b) pair per block: resident blocks overlap their phases
    const long long ab = oo * (a + (long long)v * b), ba = oo * (b + (long long)v * a);
    double *r1v = zs + 2 * o * pitch;
    if (RANK1)
        for (int k = threadIdx.x; k < 4 * o; k += blockDim.x) {
            const int w = k / o, i = k % o;
            r1v[k] = w == 0 ? t1[i + (long long)o * a] : w == 1 ? t1[i + (long long)o * b]
                   : w == 2 ? q[a + (long long)v * i] : q[b + (long long)v * i];
        }
    {
        for (int ij = threadIdx.x; ij < ooi; ij += blockDim.x) {
            const int i = ij % o, j = ij / o;
            zs[j + pitch * i] = Z[ab + ij];
            zs[o * pitch + j + pitch * i] = Z[ba + ij];
        }
        __syncthreads();
        for (int ij = threadIdx.x; ij < ooi; ij += blockDim.x) {
            const int i = ij % o, j = ij / o;
            // Z_ab[i,j] and Z_ba[j,i]; Z_ba[i,j] and Z_ab[j,i]
            const double zab = zs[j + pitch * i], zba_t = zs[o * pitch + i + pitch * j];
            const double inv = invD[ab + ij];   // D is symmetric in (a, b)
            // Z's two terms first, as the folded form sums them
            double x = L[ab + ij] + (zab + zba_t);
            // C[i,j,a,b] + C[j,i,b,a] = t1[i,a] q[b,j] + t1[j,b] q[a,i]
            if (RANK1) x += r1v[i] * r1v[3 * o + j] + r1v[o + j] * r1v[2 * o + i];
            x *= inv;
            Tn[ab + ij] = x;
            if (Told) { const double d = x - Told[ab + ij]; acc = fma(d, d, acc); }
            if (a != b) {
                const double zba = zs[o * pitch + j + pitch * i], zab_t = zs[i + pitch * j];
                double y = L[ba + ij] + (zba + zab_t);
                if (RANK1) y += r1v[o + i] * r1v[2 * o + j] + r1v[j] * r1v[3 * o + i];
                y *= inv;
                Tn[ba + ij] = y;
                if (Told) { const double d = y - Told[ba + ij]; acc = fma(d, d, acc); }
            }
        }
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}


// The finalisation from the folded ladders L = [L+ | L-] (np x nq each, np = o(o+1)/2 occupied
// pairs (i <= j), nq = v(v+1)/2 virtual pairs, pair index j(j+1)/2 + i; column q = the block's
// pair (a <= b)).  The result is pair-symmetric, Tn[i,j,a,b] = Tn[j,i,b,a], so an occupied pair
// (i0 <= j0) has two values,
//   u = (L+ + L-) + (Z_ab[i0,j0] + Z_ba[j0,i0])   -> Tn[i0,j0,a,b] and Tn[j0,i0,b,a]
//   w = (L+ - L-) + (Z_ab[j0,i0] + Z_ba[i0,j0])   -> Tn[j0,i0,a,b] and Tn[i0,j0,b,a]
// (L- = 0 for i0 = j0 or a = b; with RANK1 the rank-one pair terms at (i0,j0) and (j0,i0) too).
// All four share one denominator, invF[p + np q] = 1/D[i0,j0,a,b] (the folded 1/D).  One thread
// forms u/D and w/D from the four Z elements that it alone reads and writes them back over those
// elements in shared memory; the block then stores Tn coalesced.  Two FP64 operations per element
// of Tn (FP64 issue, at about 0.6e12 operations/s, bounds this kernel with the memory traffic).
template <bool RANK1>
__global__ void __launch_bounds__(256, RANK1 ? 6 : 8) t2_finalize_fold_kernel(const double *__restrict__ L,
                                                               const double *__restrict__ Z,
                                                               const double *__restrict__ invF, int o, int v,
                                                               const double *__restrict__ Told,
                                                               double *__restrict__ Tn, double *part,
                                                               const double *__restrict__ t1,
                                                               const double *__restrict__ q) {
    extern __shared__ double zs[];   // Z_ab then Z_ba, element (i, j) at j + pitch i; then 4 o (RANK1)
    const int pitch = o | 1;
    const long long oo = (long long)o * o;
    const int ooi = o * o, np = o * (o + 1) / 2;
    const long long nq = (long long)v * (v + 1) / 2;
    double acc = 0.0;
    int a, b;
    pair_ab32((int)blockIdx.x, a, b);
    const long long ab = oo * (a + (long long)v * b), ba = oo * (b + (long long)v * a);
    double *za = zs, *zb = zs + o * pitch, *r1v = zs + 2 * o * pitch;
    if (RANK1)
        for (int k = threadIdx.x; k < 4 * o; k += blockDim.x) {
            const int w = k / o, i = k % o;
            r1v[k] = w == 0 ? t1[i + (long long)o * a] : w == 1 ? t1[i + (long long)o * b]
                   : w == 2 ? q[a + (long long)v * i] : q[b + (long long)v * i];
        }
    for (int ij = threadIdx.x; ij < ooi; ij += blockDim.x) {
        const int i = ij % o, j = ij / o;
        za[j + pitch * i] = Z[ab + ij];
        zb[j + pitch * i] = Z[ba + ij];
    }
    __syncthreads();
    const double *lp = L + (long long)np * blockIdx.x, *lm = lp + (long long)np * nq;
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
        int i0, j0;
        pair_ab32(p, i0, j0);
        const double lpv = lp[p], lmv = (i0 == j0 || a == b) ? 0.0 : lm[p];
        const int x1 = j0 + pitch * i0, x2 = i0 + pitch * j0;   // (i0, j0) and (j0, i0)
        double u = (lpv + lmv) + (za[x1] + zb[x2]);
        double w = (lpv - lmv) + (za[x2] + zb[x1]);
        if (RANK1) {
            // C[i,j,a,b] + C[j,i,b,a] = t1[i,a] q[b,j] + t1[j,b] q[a,i]
            u += r1v[i0] * r1v[3 * o + j0] + r1v[o + j0] * r1v[2 * o + i0];
            w += r1v[j0] * r1v[3 * o + i0] + r1v[o + i0] * r1v[2 * o + j0];
        }
        const double inv = invF[p + (long long)np * blockIdx.x];
        u *= inv;
        w *= inv;
        za[x1] = u;
        zb[x2] = u;
        za[x2] = w;
        zb[x1] = w;
    }
    __syncthreads();
    for (int ij = threadIdx.x; ij < ooi; ij += blockDim.x) {
        const int i = ij % o, j = ij / o;
        const double x = za[j + pitch * i];
        Tn[ab + ij] = x;
        if (Told) { const double d = x - Told[ab + ij]; acc = fma(d, d, acc); }
        if (a != b) {
            const double y = zb[j + pitch * i];
            Tn[ba + ij] = y;
            if (Told) { const double d = y - Told[ba + ij]; acc = fma(d, d, acc); }
        }
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// Folding of a pair-symmetric contraction (the ladders, X, Y).  For an index pair (e, f) of
// extent d, q = f(f+1)/2 + e (e <= f) numbers the d(d+1)/2 pairs.  Block q writes, for every row
// r < R,
//   out+[r + R q] = c (src[ro(r) + e ke + f kf] + src[ro(r) + f ke + e kf])
//   out-[r + R q] = c (src[ro(r) + e ke + f kf] - src[ro(r) + f ke + e kf])
// (out- = out+ + R nk, nk = d(d+1)/2), c = scale, halved on the diagonal e = f when diag_half.
// Rows: with rowpair, r is itself a pair (a <= b) and ro(r) = a rs0 + b rs1; else
// ro(r) = (r mod rd) rs0 + (r / rd) rs1.
__global__ void __launch_bounds__(256) pair_fold_kernel(const double *__restrict__ src, long long R, int rowpair,
                                                        long long rd, long long rs0, long long rs1, long long ke,
                                                        long long kf, long long nk, double scale, int diag_half,
                                                        double *__restrict__ out) {
    int e, f;
    pair_ab32((int)blockIdx.x, e, f);
    const long long k1 = e * ke + f * kf, k2 = f * ke + e * kf;
    const double c = (diag_half && e == f) ? 0.5 * scale : scale;
    double *op = out + R * (long long)blockIdx.x, *om = op + R * nk;
    for (long long r = threadIdx.x; r < R; r += blockDim.x) {
        long long ro;
        if (rowpair) {
            int a, b;
            pair_ab32((int)r, a, b);
            ro = a * rs0 + b * rs1;
        } else {
            long long r1, r0;
            divmod_ll(r, rd, r1, r0);
            ro = r0 * rs0 + r1 * rs1;
        }
        const double x = src[ro + k1], y = src[ro + k2];
        if (c == 1.0) {   // FP64 issue, not memory, paces this kernel: one operation per output
            op[r] = x + y;
            om[r] = x - y;
        } else {
            op[r] = c * (x + y);
            om[r] = c * (x - y);
        }
    }
}

// The inverse for a pair index (i, j) of extent o (np = o(o+1)/2 pairs): for every i, j < o and
// column c < C,
//   out[(i + o j) sij + c sc] = base[same] + P+[p tp + c tc] + sgn P-[p tp + c tc]
// with p the pair of (min(i,j), max(i,j)), sgn = +1 for i < j, -1 for i > j, and no P- term for
// i = j (P- = P+ + npc).  ijfast: consecutive threads take consecutive (i, j), else consecutive c.
__global__ void __launch_bounds__(256) pair_unfold_kernel(const double *__restrict__ P, long long npc,
                                                          const double *__restrict__ base, int o, long long C,
                                                          long long sij, long long sc, long long tp, long long tc,
                                                          int ijfast, double *__restrict__ out) {
    const long long oo = (long long)o * o, n = oo * C;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
         x += (long long)gridDim.x * blockDim.x) {
        long long ij, c;
        if (ijfast) divmod_ll(x, oo, c, ij);
        else divmod_ll(x, C, ij, c);
        const int i = (int)(ij % o), j = (int)(ij / o);
        const int i0 = min(i, j), j0 = max(i, j);
        const long long pi = (long long)(j0 * (j0 + 1) / 2 + i0) * tp + c * tc;
        double val = P[pi];
        if (i != j) val += i < j ? P[npc + pi] : -P[npc + pi];
        const long long oi = ij * sij + c * sc;
        out[oi] = (base ? base[oi] : 0.0) + val;
    }
}

// T~[i,j,a,b] = 2 T[i,j,a,b] - T[j,i,a,b], one (a,b) block per iteration with its transpose
// through shared memory (odd row pitch), every global access unit-stride
__global__ void __launch_bounds__(256) t_tilde_smem_kernel(const double *__restrict__ T, int o, int v,
                                                           double *__restrict__ out) {
    extern __shared__ double ts[];
    const int pitch = o | 1;
    const long long oo = (long long)o * o, vv = (long long)v * v;
    const int ooi = o * o;
    for (long long ab = blockIdx.x; ab < vv; ab += gridDim.x) {
        const double *Tb = T + oo * ab;
        __syncthreads();
        for (int ij = threadIdx.x; ij < ooi; ij += blockDim.x) ts[ij / o + pitch * (ij % o)] = Tb[ij];
        __syncthreads();
        for (int ij = threadIdx.x; ij < ooi; ij += blockDim.x) {
            const int i = ij % o, j = ij / o;
            out[oo * ab + ij] = fma(2.0, ts[j + pitch * i], -ts[i + pitch * j]);
        }
    }
}

__global__ void divide_by_d_kernel(const double *__restrict__ in, const double *__restrict__ eps, int o,
                                   int v, double *__restrict__ out) {
    const long long oo = (long long)o * o, n = oo * v * v;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
         x += (long long)gridDim.x * blockDim.x) {
        long long ij = x % oo, ab = x / oo;
        int i = (int)(ij % o), j = (int)(ij / o), a = (int)(ab % v), b = (int)(ab / v);
        out[x] = in[x] / (eps[i] + eps[j] - eps[o + a] - eps[o + b]);
    }
}

__global__ void t_tilde_kernel(const double *__restrict__ T, int o, int v, double *__restrict__ out) {
    const long long oo = (long long)o * o, n = oo * v * v;
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < n;
         x += (long long)gridDim.x * blockDim.x) {
        long long ij = x % oo, ab = x - ij;
        int i = (int)(ij % o), j = (int)(ij / o);
        out[x] = 2.0 * T[x] - T[ab + j + (long long)o * i];
    }
}


// out = sum_k c_k p_k with the vector count a template parameter, so every load of an element is
// in flight at once; pairs of elements as 16-byte loads and stores (the vectors are 16-byte
// aligned), the odd last element alone.  The sum runs in k order for every element.
template <int M>
__global__ void lincomb_kernel(size_t n, VecList vl, double *__restrict__ out) {
    const size_t n2 = n / 2;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x) {
        double2 x[M];
#pragma unroll
        for (int k = 0; k < M; ++k) x[k] = __ldg(reinterpret_cast<const double2 *>(vl.p[k]) + i);
        double2 r = make_double2(0.0, 0.0);
#pragma unroll
        for (int k = 0; k < M; ++k) {
            r.x = fma(vl.c[k], x[k].x, r.x);
            r.y = fma(vl.c[k], x[k].y, r.y);
        }
        reinterpret_cast<double2 *>(out)[i] = r;
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        double r = 0.0;
#pragma unroll
        for (int k = 0; k < M; ++k) r = fma(vl.c[k], vl.p[k][n - 1], r);
        out[n - 1] = r;
    }
}

// DIIS bookkeeping of one sweep in one pass: e = xn - x (and v = xn when v_out is given), e.e (the
// same grid, products and summation order as dot_kernel, so the sum is identical) and old_k.e for
// the NOLD stored errors; row r of the partial sums at part[r gridDim.x + block].  The sweep
// writes xn into its DIIS slot itself, so v_out is null there.
template <int NOLD>
__global__ void diis_pair_dots_kernel(size_t n, const double *__restrict__ xn, const double *__restrict__ x,
                                      double *__restrict__ v_out, double *__restrict__ e_out, VecList olds,
                                      double *part) {
    double acc = 0.0, accs[NOLD > 0 ? NOLD : 1];
#pragma unroll
    for (int k = 0; k < NOLD; ++k) accs[k] = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double xv = xn[i];
        const double e = xv - x[i];
        if (v_out) v_out[i] = xv;
        e_out[i] = e;
        acc = fma(e, e, acc);
#pragma unroll
        for (int k = 0; k < NOLD; ++k) accs[k] = fma(__ldg(olds.p[k] + i), e, accs[k]);
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
#pragma unroll
    for (int k = 0; k < NOLD; ++k) {
        const double v = block_sum(accs[k]);
        if (threadIdx.x == 0) part[(size_t)(1 + k) * gridDim.x + blockIdx.x] = v;
    }
}

// out[b] = sum of row b of part (rows of n), in reduce_partials' order
__global__ void reduce_rows(const double *part, int n, double *out) {
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[(size_t)blockIdx.x * n + i];
    v = block_sum(v);
    if (threadIdx.x == 0) out[blockIdx.x] = v;
}

// W'[(m,n),(i,j)] -= [m = i] Fmi[n,j] (first = true) or [n = j] Fmi[m,i]: the two Fmi terms of
// the T2 update ride in the hole-hole ladder.  One thread per (i, j, k); within one launch every
// entry has one writer, and the two launches are ordered on the stream.
__global__ void wp_fmi_kernel(double *__restrict__ Wp, const double *__restrict__ Fmi, int o, bool first) {
    const long long oo = (long long)o * o, ooo = oo * o;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ooo;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % o);
        const long long ij = t / o;
        const int i = (int)(ij % o), j = (int)(ij / o);
        if (first)
            Wp[oo * ij + i + (long long)o * k] -= Fmi[k + (long long)o * j];   // m = i, n = k
        else
            Wp[oo * ij + k + (long long)o * j] -= Fmi[k + (long long)o * i];   // m = k, n = j
    }
}

// Fmi[m,i] = sum_n 2 X[m,n,i,n] - X[m,n,n,i] with X = W' - oooo, W'[(m,n),(i,j)] = oooo + sum_ef
// oovv[m,n,e,f] T[i,j,e,f]: the Fmi contraction of RCCD.jl:216 (sum_nef oovv[m,n,e,f] T~[i,n,e,f])
// read off the hole-hole intermediate instead of a GEMM of its own.  One warp per (m, i), its
// lanes over n.
__global__ void fmi_from_x_kernel(const double *__restrict__ Wp, const double *__restrict__ oooo, int o,
                                  double *__restrict__ Fmi) {
    const long long oo = (long long)o * o;
    const long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= oo) return;
    const int m = (int)(t % o), i = (int)(t / o);
    double acc = 0.0;
    for (int n = lane; n < o; n += 32) {
        const long long mn = m + (long long)o * n;
        const long long d = mn + oo * (i + (long long)o * n), x = mn + oo * (n + (long long)o * i);
        acc = fma(2.0, Wp[d] - oooo[d], acc);
        acc -= Wp[x] - oooo[x];
    }
    acc = warp_allsum(acc);
    if (lane == 0) Fmi[t] = acc;
}

// Fae from the ring intermediates and the Fae term folded into W12.  With t = WJ - J0 and
// u = WK - K0 (the GEMM parts of WmBeJ and WmBEj, layout [(m,e),(b,j)]), their traces
// tJ[a,e] = sum_m t[(m,e),(a,m)] and tK[a,e] = sum_m u[(m,e),(a,m)] (the seeds' traces trJ0, trK0
// formed once) give
// Fae[a,e] = -(cJ tJ + cK tK) by the pair symmetry of T2; then W12[(j,e),(a,j)] += Fae[a,e]
// for every j, so the ring GEMM T[i,m,a,e] W12[(m,e),(b,j)] also yields T[i,j,a,e] Fae[b,e].
// One warp per (a, e), its lanes over m; the (m = j) entries it reads and the ones it updates
// are the same.
__global__ void fae_trace_kernel(const double *__restrict__ WJ, const double *__restrict__ trJ0,
                                 const double *__restrict__ WK, const double *__restrict__ trK0, int o, int v,
                                 double cJ, double cK, double *__restrict__ Fae, double *__restrict__ W12) {
    const long long ov = (long long)o * v;
    const long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= (long long)v * v) return;
    const int e = (int)(t % v), a = (int)(t / v);
    const long long base = (long long)o * e + ov * a, step = 1 + ov * v;
    double tj = 0.0, tk = 0.0;
    for (int m = lane; m < o; m += 32) {
        const long long x = base + step * m;
        tj += WJ[x];
        tk += WK[x];
    }
    const long long ae = a + (long long)v * e;
    const double f = -(cJ * (warp_allsum(tj) - trJ0[ae]) + cK * (warp_allsum(tk) - trK0[ae]));
    if (lane == 0) Fae[a + (long long)v * e] = f;
    if (W12)
        for (int j = lane; j < o; j += 32) W12[base + step * j] += f;
}

// CCSD sweep inputs from T2 and t1 in one pass: Ttau = T2 + tau and U = T2 + 2 tau with
// tau[i,j,a,b] = t1[i,a] t1[j,b]; an elementwise grid-stride pass (32-bit indices, t1 from L1).
__global__ void __launch_bounds__(256) ccsd_tau_kernel(const double *__restrict__ T, const double *__restrict__ t1,
                                                       unsigned o, unsigned v, unsigned n, double *__restrict__ Ttau,
                                                       double *__restrict__ U) {
    const unsigned oo = o * o;
    for (unsigned x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
        const unsigned ij = x % oo, ab = x / oo;
        const unsigned i = ij % o, j = ij / o, a = ab % v, b = ab / v;
        const double t = T[x], tau = __ldg(t1 + i + o * a) * __ldg(t1 + j + o * b);
        Ttau[x] = t + tau;
        U[x] = fma(2.0, tau, t);
    }
}

// Traces over m of the GEMM parts of the ring intermediates (layout [(m,e),(b,j)]):
// tJ[a,e] = sum_m WJ[(m,e),(a,m)] - trJ0[a,e], tK likewise (null trJ0, trK0: the plain traces,
// which is how the seeds' traces are formed once).  One thread
// warp per (a, e), its lanes over m.
__global__ void ring_traces_kernel(const double *__restrict__ WJ, const double *__restrict__ trJ0,
                                   const double *__restrict__ WK, const double *__restrict__ trK0, int o, int v,
                                   double *__restrict__ tJ, double *__restrict__ tK) {
    const long long ov = (long long)o * v;
    const long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= (long long)v * v) return;
    const int e = (int)(t % v), a = (int)(t / v);
    const long long base = (long long)o * e + ov * a, step = 1 + ov * v;
    double tj = 0.0, tk = 0.0;
    for (int m = lane; m < o; m += 32) {
        const long long x = base + step * m;
        tj += WJ[x];
        tk += WK[x];
    }
    tj = warp_allsum(tj);
    tk = warp_allsum(tk);
    const long long ae = a + (long long)v * e;
    if (lane == 0) {
        tJ[ae] = tj - (trJ0 ? trJ0[ae] : 0.0);
        tK[ae] = tk - (trK0 ? trK0[ae] : 0.0);
    }
}

// CCSD Fae and F~ae from the ring intermediates (RCCSD.jl:187-194, or mRCCSD.jl:137-149's t1
// term).  With the traces tGJ, tGK of the T2 parts of WmBeJ / WmBEj (taken before their t1
// terms) and tJ, tK of the complete ones (this kernel, after), and the pair symmetry of T2:
//   H1[a,e] = sum_mf t1[m,f] <ma|ef> = tJ - tGJ + S1,   G2[a,e] = sum_mf t1[m,f] <ma|fe> = tGK - tK + S2,
// S1[a,e] = sum_n t1[n,a] c1[n,e], S2[a,e] = sum_n t1[n,a] c2[n,e] (the traces of the ooov t1
// terms, c1[n,e] = sum_m ooov[n,m,m,e], c2[n,e] = sum_m ooov[m,n,m,e]), and
//   Fae = 2 G2 - H1' - (tGJ + 2 tGK) + 1/2 t1^T (Fme - fOV) + fVV - 1/2 t1^T fOV
// (H1' = H1, or H1^T for mRCCSD.jl:140's <me|af>), F~ae = Fae - 1/2 t1^T Fme.  Writes Fae, H1, G2
// (the T1 equation's tau corrections) and adds F~ae[a,e] to W12[(j,e),(a,j)] for every j, where
// the first ring GEMM turns it into the T2[i,j,a,e] F~ae[b,e] term.  One warp per (a, e), its
// lanes over m and n.
__global__ void ccsd_fae_kernel(const double *__restrict__ WJ, const double *__restrict__ trJ0,
                                const double *__restrict__ WK, const double *__restrict__ trK0,
                                const double *__restrict__ tGJ, const double *__restrict__ tGK,
                                const double *__restrict__ t1, const double *__restrict__ c12,
                                const double *__restrict__ Fme, const double *__restrict__ fOV,
                                const double *__restrict__ fVV, int o, int v, int mvariant,
                                double *__restrict__ Fae, double *__restrict__ H1, double *__restrict__ G2,
                                double *__restrict__ W12) {
    const long long ov = (long long)o * v;
    const long long t = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= (long long)v * v) return;
    const int e = (int)(t % v), a = (int)(t / v);
    const long long step = 1 + ov * v;
    const long long base = (long long)o * e + ov * a;
    const double *c1 = c12, *c2 = c12 + ov;
    double tj = 0.0, tk = 0.0, s1 = 0.0, s2 = 0.0, tf = 0.0, tfo = 0.0, tj2 = 0.0, s12 = 0.0;
    const long long base2 = (long long)o * a + ov * e;
    for (int m = lane; m < o; m += 32) {
        const long long x = base + step * m;
        tj += WJ[x];
        tk += WK[x];
        const double ta = t1[m + (long long)o * a];
        s1 = fma(ta, c1[m + (long long)o * e], s1);
        s2 = fma(ta, c2[m + (long long)o * e], s2);
        tf = fma(ta, Fme[m + (long long)o * e], tf);
        if (fOV) tfo = fma(ta, fOV[m + (long long)o * e], tfo);
        if (mvariant) {
            // H1[e,a]: the WJ trace at [(m,a),(e,m)] and S1[e,a]
            tj2 += WJ[base2 + step * m];
            s12 = fma(t1[m + (long long)o * e], c1[m + (long long)o * a], s12);
        }
    }
    const long long ae = a + (long long)v * e, ea = e + (long long)v * a;
    tj = warp_allsum(tj) - trJ0[ae]; tk = warp_allsum(tk) - trK0[ae]; s1 = warp_allsum(s1); s2 = warp_allsum(s2);
    tf = warp_allsum(tf); tfo = warp_allsum(tfo);
    if (mvariant) { tj2 = warp_allsum(tj2) - trJ0[ea]; s12 = warp_allsum(s12); }
    const double h1 = tj - tGJ[ae] + s1, g2 = tGK[ae] - tk + s2;
    const double h1x = mvariant ? tj2 - tGJ[e + (long long)v * a] + s12 : h1;
    double ft = 2.0 * g2 - h1x - (tGJ[ae] + 2.0 * tGK[ae]) - tfo;   // F~ae
    if (fVV) ft += fVV[ae];
    if (lane == 0) {
        Fae[ae] = fma(0.5, tf, ft);
        H1[ae] = h1;
        G2[ae] = g2;
    }
    for (int j = lane; j < o; j += 32) W12[base + step * j] += ft;
}

// T1's <ma|fe> terms from Y[(i,j),(a,m)] = sum_ef Ttau[i,j,e,f] <ma|fe> (the Wabef t1
// intermediate, RCCSD.jl:256-257 / mRCCSD.jl:210-211):
//   R1[i,a] += 2 (sum_m Y[(i,m),(a,m)] - sum_e t1[i,e] G2[a,e]) - (sum_m Y[(m,i),(a,m)] - sum_f t1[i,f] H1[a,f])
// (the tau parts of Ttau removed through G2 and H1).  One thread per (i, a).
__global__ void t1_ytrace_kernel(const double *__restrict__ Y, const double *__restrict__ t1,
                                 const double *__restrict__ G2, const double *__restrict__ H1,
                                 const double *__restrict__ c123, int o, int v, double *__restrict__ R1) {
    const long long oo = (long long)o * o;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)o * v) return;
    const int i = (int)(t % o), a = (int)(t / o);
    double y1 = 0.0, y2 = 0.0;
    for (int m = 0; m < o; ++m) {
        const long long col = oo * (a + (long long)v * m);
        y1 += Y[i + (long long)o * m + col];
        y2 += Y[m + (long long)o * i + col];
    }
    // Y carries its ooov seed Q0[i,j,a,m] = ooov[m,i,j,a], whose traces are c2[i,a] and c3[i,a]
    const long long ov = (long long)o * v;
    y1 -= c123[ov + t];
    y2 -= c123[2 * ov + t];
    double g = 0.0, h = 0.0;
    for (int e = 0; e < v; ++e) {
        const double te = t1[i + (long long)o * e];
        g = fma(te, G2[a + (long long)v * e], g);
        h = fma(te, H1[a + (long long)v * e], h);
    }
    R1[t] += 2.0 * (y1 - g) - (y2 - h);
}

// T1's Fme term, R1[i,a] += sum_{m,e} (2 T2[i,m,a,e] - T2[m,i,a,e]) Fme[m,e], in one read of T2: block
// (a, chunk) takes the o x o blocks T2[:,:,a,e] of its e range through shared memory (odd pitch for
// the transposed reads) and writes its per-i sums to part[chunk][i + o a]; o <= 64.
constexpr int T1FME_CHUNK = 8;
__global__ void __launch_bounds__(256) t1_fme_kernel(const double *__restrict__ T, const double *__restrict__ Fme,
                                                     int o, int v, double *__restrict__ part) {
    extern __shared__ double tile[];   // [o][pitch], element (i, m) of the block at i + pitch m
    __shared__ double fm[64];          // Fme[:, e]
    const int pitch = o | 1, ooi = o * o;
    const int a = blockIdx.x, chunk = blockIdx.y;
    const long long oo = (long long)o * o;
    // thread (i, g): row i, quarter g of the m range (o <= 64: four groups of 64 threads)
    const int i = threadIdx.x & 63, g = threadIdx.x >> 6;
    double acc = 0.0;
    const int e0 = chunk * T1FME_CHUNK, e1 = min(v, e0 + T1FME_CHUNK);
    for (int e = e0; e < e1; ++e) {
        const double *blk = T + oo * (a + (long long)v * e);
        __syncthreads();
        for (int im = threadIdx.x; im < ooi; im += blockDim.x) tile[(im % o) + pitch * (im / o)] = blk[im];
        if (threadIdx.x < o) fm[threadIdx.x] = Fme[threadIdx.x + (long long)o * e];
        __syncthreads();
        if (i < o)
            for (int m = g; m < o; m += 4) acc = fma(2.0 * tile[i + pitch * m] - tile[m + pitch * i], fm[m], acc);
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    if (g == 0 && i < o)
        part[(long long)chunk * o * v + i + (long long)o * a] = red[i] + red[i + 64] + red[i + 128] + red[i + 192];
}

// R1[x] += sum over chunks of part[chunk][x], in chunk order
__global__ void t1_fme_reduce_kernel(const double *__restrict__ part, int nchunk, long long n, double *__restrict__ R1) {
    const long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (x >= n) return;
    double s = 0.0;
    for (int c = 0; c < nchunk; ++c) s += part[c * n + x];
    R1[x] += s;
}

// c1[n,e] = sum_m ooov[n,m,m,e], c2[n,e] = sum_m ooov[m,n,m,e], c3[n,e] = sum_m ooov[m,m,n,e]
// (ooov column-major o x o x o x v)
__global__ void ooov_diag_sums_kernel(const double *__restrict__ ooov, int o, int v, double *__restrict__ c12) {
    const long long oo = (long long)o * o, ooo = oo * o, ov = (long long)o * v;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= ov) return;
    const int n = (int)(t % o), e = (int)(t / o);
    double s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (int m = 0; m < o; ++m) {
        s1 += ooov[n + (long long)o * m + oo * m + ooo * e];
        s2 += ooov[m + (long long)o * n + oo * m + ooo * e];
        s3 += ooov[m + (long long)o * m + oo * n + ooo * e];
    }
    c12[t] = s1;
    c12[ov + t] = s2;
    c12[2 * ov + t] = s3;
}

__global__ void t1_finalize_kernel(double *__restrict__ t1n, const double *__restrict__ eps, int o, int v,
                                   const double *__restrict__ t1old, double *part) {
    double acc = 0.0;
    const long long n = (long long)o * v;
    for (long long x = threadIdx.x; x < n; x += blockDim.x) {
        int i = (int)(x % o), a = (int)(x / o);
        double val = t1n[x] / (eps[i] - eps[o + a]);
        t1n[x] = val;
        if (t1old) { double d = val - t1old[x]; acc = fma(d, d, acc); }
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[0] = acc;
}

// MP2 adjoint seed from chemists' K[i,a,j,b]: Gamma = 2 e_bar (2K_iajb - K_ibja)/D and the energy
__global__ void mp2_gamma_kernel(const double *__restrict__ K, const double *__restrict__ eps, int o, int v,
                                 double e_bar, double *__restrict__ G, double *part) {
    const long long ov = (long long)o * v, oo = (long long)o * o;
    const long long npair = (long long)v * (v + 1) / 2;
    double acc = 0.0;
    for (long long p = blockIdx.x; p < npair; p += gridDim.x) {
        int a, b;
        pair_ab(p, a, b);
        const double ea = eps[o + a], eb = eps[o + b];
        for (long long ij = threadIdx.x; ij < oo; ij += blockDim.x) {
            const int i = (int)(ij % o), j = (int)(ij / o);
            const long long x_off = i + (long long)o * a + ov * j + ov * o * b;   // K[i,a,j,b]
            const long long y_off = i + (long long)o * b + ov * j + ov * o * a;   // K[i,b,j,a]
            const double inv = 1.0 / (eps[i] + eps[j] - ea - eb);
            const double x = K[x_off];
            if (a == b) {
                acc = fma(x * x, inv, acc);
                if (G) G[x_off] = 2.0 * e_bar * x * inv;
            } else {
                const double y = K[y_off];
                acc = fma(x * (2.0 * x - y) + y * (2.0 * y - x), inv, acc);
                if (G) {
                    G[x_off] = 2.0 * e_bar * (2.0 * x - y) * inv;
                    G[y_off] = 2.0 * e_bar * (2.0 * y - x) * inv;
                }
            }
        }
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

unsigned grid_for(long long n, int threads = 256) {
    long long b = (n + threads - 1) / threads;
    if (b > 152LL * 32) b = 152LL * 32;
    if (b < 1) b = 1;
    return (unsigned)b;
}

double finish_reduce(Ctx *ctx, int nblocks) {
    reduce_partials<<<1, 1024, 0, ctx->stream>>>(ctx->d_red, nblocks, ctx->d_red + 65536 - 8);
    ctx->count_launch();
    JUES_CHECK_CUDA(cudaGetLastError());
    double h = 0.0;
    JUES_CHECK_CUDA(cudaMemcpyAsync(&h, ctx->d_red + 65536 - 8, sizeof(double), cudaMemcpyDeviceToHost,
                                    ctx->stream));
    JUES_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    return h;
}

}  // namespace

void permute4(Ctx *ctx, const Perm4 &p, double alpha, const double *in, double beta, double *out) {
    long long total = p.d[0] * p.d[1] * p.d[2] * p.d[3];
    if (total == 0) return;
    Ctx::Scope s(ctx, "permute4");
    // the input's and the output's unit-stride dimensions (extent > 1)
    int ki = -1, ko = -1;
    for (int k = 0; k < 4; ++k) {
        if (p.d[k] > 1 && p.si[k] == 1 && ki < 0) ki = k;
        if (p.d[k] > 1 && p.so[k] == 1 && ko < 0) ko = k;
    }
    if (ki < 0 || ko < 0 || ki == ko) {
        // both sides are coalesced along the same dimension (or neither has a unit stride)
        permute4_kernel<<<grid_for(total), 256, 0, ctx->stream>>>(p, alpha, in, beta, out, total);
        JUES_CHECK_CUDA(cudaGetLastError());
        return;
    }
    int rest[2], nr = 0;
    for (int k = 0; k < 4; ++k)
        if (k != ki && k != ko) rest[nr++] = k;
    const long long tiles = ((p.d[ki] + 31) / 32) * ((p.d[ko] + 31) / 32);
    JUES_REQUIRE(tiles < (1LL << 31), "permutation too large");
    const long long nrest = p.d[rest[0]] * p.d[rest[1]];
    const unsigned gy = (unsigned)std::min<long long>(nrest, std::max<long long>(1, 152LL * 32 / std::max(1LL, tiles)) * 8);
    // 16-byte accesses need even extents and strides along the tile and 16-byte aligned bases
    bool vec = p.d[ki] % 2 == 0 && p.d[ko] % 2 == 0 && (reinterpret_cast<uintptr_t>(in) & 15) == 0 &&
               (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    for (int k = 0; k < 4; ++k)
        if (k != ki) vec = vec && p.si[k] % 2 == 0;
    for (int k = 0; k < 4; ++k)
        if (k != ko) vec = vec && p.so[k] % 2 == 0;
    const dim3 grid((unsigned)tiles, std::max(1u, gy)), block(32, 8);
    if (vec)
        permute4_tiled_kernel<true><<<grid, block, 0, ctx->stream>>>(p, ki, ko, rest[0], rest[1], alpha, in, beta, out);
    else
        permute4_tiled_kernel<false><<<grid, block, 0, ctx->stream>>>(p, ki, ko, rest[0], rest[1], alpha, in, beta, out);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void fill(Ctx *ctx, double *p, size_t n, double v) {
    if (!n) return;
    Ctx::Scope s(ctx, "fill");
    fill_kernel<<<grid_for((long long)n), 256, 0, ctx->stream>>>(p, n, v);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void axpby(Ctx *ctx, size_t n, double a, const double *x, double b, const double *y, double *out) {
    if (!n) return;
    Ctx::Scope s(ctx, "axpby");
    axpby_kernel<<<grid_for((long long)n), 256, 0, ctx->stream>>>(n, a, x, b, y, out);
    JUES_CHECK_CUDA(cudaGetLastError());
}

double dot(Ctx *ctx, size_t n, const double *x, const double *y) {
    {
        Ctx::Scope s(ctx, "dot");
        dot_kernel<<<RED_BLOCKS, RED_THREADS, 0, ctx->stream>>>(n, x, y, ctx->d_red);
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    return finish_reduce(ctx, RED_BLOCKS);
}

bool any_nonfinite(Ctx *ctx, const double *x, size_t n) {
    if (!n) return false;
    JUES_CHECK_CUDA(cudaMemsetAsync(ctx->d_flags + 1, 0, sizeof(unsigned), ctx->stream));
    {
        Ctx::Scope s(ctx, "nonfinite");
        nonfinite_kernel<<<grid_for((long long)n), 256, 0, ctx->stream>>>(n, x, ctx->d_flags + 1);
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    unsigned h = 0;
    JUES_CHECK_CUDA(cudaMemcpyAsync(&h, ctx->d_flags + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    JUES_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    return h != 0;
}

double mp2_energy(Ctx *ctx, const double *K, const double *eps, int o, int v) {
    long long npair = (long long)v * (v + 1) / 2;
    int nb = (int)(npair < RED_BLOCKS ? npair : RED_BLOCKS);
    if (nb < 1) return 0.0;
    {
        Ctx::Scope s(ctx, "mp2_energy");
        mp2_kernel<<<nb, RED_THREADS, 0, ctx->stream>>>(K, eps, o, v, ctx->d_red);
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    return finish_reduce(ctx, nb);
}

double mp2_gamma(Ctx *ctx, const double *K, const double *eps, int o, int v, double e_bar, double *G) {
    long long npair = (long long)v * (v + 1) / 2;
    int nb = (int)(npair < RED_BLOCKS ? npair : RED_BLOCKS);
    {
        Ctx::Scope s(ctx, "mp2_gamma");
        mp2_gamma_kernel<<<nb, RED_THREADS, 0, ctx->stream>>>(K, eps, o, v, e_bar, G, ctx->d_red);
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    return finish_reduce(ctx, nb);
}

double cc_energy(Ctx *ctx, const double *oovv, const double *T2, const double *t1, int o, int v) {
    long long vv = (long long)v * v;
    int nb = (int)(vv < RED_BLOCKS ? vv : RED_BLOCKS);
    if (nb < 1) return 0.0;
    {
        Ctx::Scope s(ctx, "cc_energy");
        ccenergy_kernel<<<nb, RED_THREADS, 0, ctx->stream>>>(oovv, T2, t1, o, v, ctx->d_red);
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    return finish_reduce(ctx, nb);
}

void inv_denominators_folded(Ctx *ctx, const double *eps, int o, int v, double *out) {
    const long long n = (long long)o * (o + 1) / 2 * ((long long)v * (v + 1) / 2);
    JUES_REQUIRE(o * (o + 1) / 2 < (1 << 26) && (long long)v * (v + 1) / 2 < (1LL << 26), "folded 1/D: too large");
    Ctx::Scope s(ctx, "inv_denominators");
    inv_denominators_folded_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(eps, o, v, out);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void inv_denominators(Ctx *ctx, const double *eps, int o, int v, double *out) {
    long long n = (long long)o * o * v * v;
    Ctx::Scope s(ctx, "inv_denominators");
    inv_denominators_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(eps, o, v, out);
    JUES_CHECK_CUDA(cudaGetLastError());
}

bool t2_finalize_folds(int o, int v) { return o <= 64 && (long long)v * (v + 1) / 2 <= 65536 - 64; }

double t2_finalize(Ctx *ctx, const double *L, const double *Z, const double *invD, int o, int v,
                   const double *Told, double *Tn, const double *t1, const double *q, bool pairl) {
    JUES_REQUIRE(!t1 == !q, "t2_finalize: t1 and q come together");
    JUES_REQUIRE(!pairl || t2_finalize_folds(o, v), "t2_finalize: folded ladders need nocc <= 64, nvir <= 361");
    long long npair = (long long)v * (v + 1) / 2;
    int nb = (int)(npair < RED_BLOCKS ? npair : RED_BLOCKS);
    {
        Ctx::Scope s(ctx, "t2_finalize");
        // one block per pair; the step norm's partials (one per block) must fit the reduction scratch
        if (t2_finalize_folds(o, v)) {
            const size_t smem = ((size_t)2 * o * (o | 1) + (t1 ? 4 * o : 0)) * sizeof(double);
            // the rank-one term is a template parameter: without it the kernel fits 32 registers
            // and eight blocks per SM
            static std::atomic<unsigned long long> attr_set{0};
            const unsigned long long bit = ctx->device >= 0 && ctx->device < 64 ? 1ull << ctx->device : 0ull;
            if (smem > 48 * 1024 && (!bit || !(attr_set.load() & bit))) {
                const int most = (2 * 64 * 65 + 4 * 64) * 8;   // o = 64 with the rank-one term
                JUES_CHECK_CUDA(cudaFuncSetAttribute(t2_finalize_smem_kernel<false>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, most));
                JUES_CHECK_CUDA(cudaFuncSetAttribute(t2_finalize_smem_kernel<true>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, most));
                JUES_CHECK_CUDA(cudaFuncSetAttribute(t2_finalize_fold_kernel<false>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, most));
                JUES_CHECK_CUDA(cudaFuncSetAttribute(t2_finalize_fold_kernel<true>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, most));
                attr_set.fetch_or(bit);
            }
            nb = (int)npair;
            auto kern = t1 ? (pairl ? t2_finalize_fold_kernel<true> : t2_finalize_smem_kernel<true>)
                           : (pairl ? t2_finalize_fold_kernel<false> : t2_finalize_smem_kernel<false>);
            kern<<<nb, RED_THREADS, smem, ctx->stream>>>(L, Z, invD, o, v, Told, Tn, ctx->d_red, t1, q);
        } else {
            t2_finalize_kernel<<<nb, RED_THREADS, 0, ctx->stream>>>(L, Z, invD, o, v, Told, Tn, ctx->d_red, t1, q);
        }
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    return Told ? finish_reduce(ctx, nb) : 0.0;
}


void pair_fold(Ctx *ctx, const double *src, long long R, bool rowpair, long long rd, long long rs0, long long rs1,
               int d, long long ke, long long kf, double scale, bool diag_half, double *out) {
    const long long nk = (long long)d * (d + 1) / 2;
    JUES_REQUIRE(d > 0 && R > 0 && nk < (1LL << 26) && (!rowpair || R < (1LL << 26)), "pair_fold: bad extents");
    Ctx::Scope s(ctx, "pair_fold");
    pair_fold_kernel<<<(unsigned)nk, 256, 0, ctx->stream>>>(src, R, rowpair ? 1 : 0, rd, rs0, rs1, ke, kf, nk, scale,
                                                            diag_half ? 1 : 0, out);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void pair_unfold(Ctx *ctx, const double *P, long long npc, const double *base, int o, long long C, long long sij,
                 long long sc, long long tp, long long tc, bool ijfast, double *out) {
    const long long n = (long long)o * o * C;
    Ctx::Scope s(ctx, "pair_unfold");
    pair_unfold_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(P, npc, base, o, C, sij, sc, tp, tc, ijfast ? 1 : 0,
                                                             out);
    JUES_CHECK_CUDA(cudaGetLastError());
}

double t1_finalize(Ctx *ctx, double *t1n, const double *eps, int o, int v, const double *t1old) {
    {
        Ctx::Scope s(ctx, "t1_finalize");
        t1_finalize_kernel<<<1, 1024, 0, ctx->stream>>>(t1n, eps, o, v, t1old, ctx->d_red);
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    return t1old ? finish_reduce(ctx, 1) : 0.0;
}

void divide_by_d(Ctx *ctx, const double *in, const double *eps, int o, int v, double *out) {
    long long n = (long long)o * o * v * v;
    Ctx::Scope s(ctx, "divide_by_d");
    divide_by_d_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(in, eps, o, v, out);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void t_tilde(Ctx *ctx, const double *T, int o, int v, double *out) {
    long long n = (long long)o * o * v * v;
    Ctx::Scope s(ctx, "t_tilde");
    if (o <= 64) {
        const size_t smem = (size_t)o * (o | 1) * sizeof(double);   // <= 33 KB
        const long long vv = (long long)v * v;
        t_tilde_smem_kernel<<<(unsigned)std::min<long long>(vv, 152LL * 16), 256, smem, ctx->stream>>>(T, o, v, out);
    } else {
        t_tilde_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(T, o, v, out);
    }
    JUES_CHECK_CUDA(cudaGetLastError());
}

void diis_error(Ctx *ctx, size_t n, const double *xn, const double *x, double *v_out, double *e_out, int nold,
                const double *const *olds, double *dots) {
    JUES_REQUIRE(nold >= 0 && nold <= 15, "diis_error supports up to 15 stored errors");
    // partial sums: row 0 = e.e, rows 1..nold = old_k.e, in one pass
    {
        VecList vl;
        for (int k = 0; k < nold; ++k) { vl.p[k] = olds[k]; vl.c[k] = 0.0; }
        Ctx::Scope s(ctx, "diis_error");
        double *part = ctx->d_red;
        switch (nold) {
#define JUES_DIIS_DOTS(K) \
    case K: diis_pair_dots_kernel<K><<<RED_BLOCKS, RED_THREADS, 0, ctx->stream>>>(n, xn, x, v_out, e_out, vl, part); break;
            JUES_DIIS_DOTS(0) JUES_DIIS_DOTS(1) JUES_DIIS_DOTS(2) JUES_DIIS_DOTS(3) JUES_DIIS_DOTS(4)
            JUES_DIIS_DOTS(5) JUES_DIIS_DOTS(6) JUES_DIIS_DOTS(7) JUES_DIIS_DOTS(8) JUES_DIIS_DOTS(9)
            JUES_DIIS_DOTS(10) JUES_DIIS_DOTS(11) JUES_DIIS_DOTS(12) JUES_DIIS_DOTS(13) JUES_DIIS_DOTS(14)
            JUES_DIIS_DOTS(15)
#undef JUES_DIIS_DOTS
        }
        JUES_CHECK_CUDA(cudaGetLastError());
    }
    double *out = ctx->d_red + 65536 - 48;   // (nold + 1) <= 16 sums, clear of finish_reduce's slot
    reduce_rows<<<nold + 1, 1024, 0, ctx->stream>>>(ctx->d_red, RED_BLOCKS, out);
    ctx->count_launch();
    JUES_CHECK_CUDA(cudaGetLastError());
    JUES_CHECK_CUDA(cudaMemcpyAsync(dots, out, (nold + 1) * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    JUES_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
}

void wp_fmi(Ctx *ctx, double *Wp, const double *Fmi, int o) {
    Ctx::Scope s(ctx, "wp_fmi");
    const long long n = (long long)o * o * o;
    wp_fmi_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(Wp, Fmi, o, true);
    wp_fmi_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(Wp, Fmi, o, false);
    ctx->count_launch();
    JUES_CHECK_CUDA(cudaGetLastError());
}

void fmi_from_x(Ctx *ctx, const double *Wp, const double *oooo, int o, double *Fmi) {
    Ctx::Scope s(ctx, "fmi_trace");
    const long long n = (long long)o * o;
    fmi_from_x_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, ctx->stream>>>(Wp, oooo, o, Fmi);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void fae_from_rings(Ctx *ctx, const double *WJ, const double *trJ0, const double *WK, const double *trK0, int o,
                    int v, double cJ, double cK, double *Fae, double *W12) {
    Ctx::Scope s(ctx, "fae_trace");
    const long long n = (long long)v * v;
    fae_trace_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, ctx->stream>>>(WJ, trJ0, WK, trK0, o, v, cJ, cK, Fae,
                                                                               W12);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void ccsd_tau(Ctx *ctx, const double *T, const double *t1, int o, int v, double *Ttau, double *U) {
    const long long n = (long long)o * o * v * v;
    JUES_REQUIRE(n < (1LL << 31), "ccsd_tau: o^2 v^2 must be below 2^31");
    Ctx::Scope s(ctx, "ccsd_tau");
    ccsd_tau_kernel<<<grid_for(n), 256, 0, ctx->stream>>>(T, t1, (unsigned)o, (unsigned)v, (unsigned)n, Ttau, U);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void ring_traces(Ctx *ctx, const double *WJ, const double *trJ0, const double *WK, const double *trK0, int o, int v,
                 double *tJ, double *tK) {
    Ctx::Scope s(ctx, "fae_trace");
    const long long n = (long long)v * v;
    ring_traces_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, ctx->stream>>>(WJ, trJ0, WK, trK0, o, v, tJ, tK);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void ccsd_fae(Ctx *ctx, const double *WJ, const double *trJ0, const double *WK, const double *trK0, const double *tGJ,
              const double *tGK, const double *t1, const double *c12, const double *Fme, const double *fOV,
              const double *fVV, int o, int v, bool mvariant, double *Fae, double *H1, double *G2, double *W12) {
    Ctx::Scope s(ctx, "fae_trace");
    const long long n = (long long)v * v;
    ccsd_fae_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, ctx->stream>>>(WJ, trJ0, WK, trK0, tGJ, tGK, t1, c12, Fme,
                                                                          fOV, fVV, o, v, mvariant ? 1 : 0, Fae,
                                                                          H1, G2, W12);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void t1_ytrace(Ctx *ctx, const double *Y, const double *t1, const double *G2, const double *H1, const double *c123,
               int o, int v, double *R1) {
    Ctx::Scope s(ctx, "ccsd_t1");
    const long long n = (long long)o * v;
    t1_ytrace_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(Y, t1, G2, H1, c123, o, v, R1);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void t1_fme(Ctx *ctx, const double *T, const double *Fme, int o, int v, double *R1) {
    JUES_REQUIRE(o <= 64, "t1_fme: nocc <= 64");
    const int nchunk = (v + T1FME_CHUNK - 1) / T1FME_CHUNK;
    const long long n = (long long)o * v;
    double *part = static_cast<double *>(ctx->splitk_scratch((size_t)nchunk * n * sizeof(double)));
    Ctx::Scope s(ctx, "ccsd_t1");
    t1_fme_kernel<<<dim3((unsigned)v, (unsigned)nchunk), 256, (size_t)o * (o | 1) * sizeof(double), ctx->stream>>>(
        T, Fme, o, v, part);
    t1_fme_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(part, nchunk, n, R1);
    ctx->count_launch();
    JUES_CHECK_CUDA(cudaGetLastError());
}

void ooov_diag_sums(Ctx *ctx, const double *ooov, int o, int v, double *c12) {
    Ctx::Scope s(ctx, "ooov_diag_sums");
    const long long n = (long long)o * v;
    ooov_diag_sums_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(ooov, o, v, c12);
    JUES_CHECK_CUDA(cudaGetLastError());
}

void lincomb(Ctx *ctx, size_t n, int m, const double *const *vecs, const double *c, double *out) {
    JUES_REQUIRE(m >= 1 && m <= 16, "lincomb supports 1..16 vectors");
    VecList vl;
    for (int k = 0; k < m; ++k) { vl.p[k] = vecs[k]; vl.c[k] = c[k]; }
    bool aligned = (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    for (int k = 0; k < m; ++k) aligned = aligned && (reinterpret_cast<uintptr_t>(vecs[k]) & 15) == 0;
    JUES_REQUIRE(aligned, "lincomb: vectors must be 16-byte aligned");
    Ctx::Scope s(ctx, "lincomb");
    const unsigned grid = grid_for((long long)(n / 2 + 1));
    switch (m) {
#define JUES_LINCOMB(K) \
    case K: lincomb_kernel<K><<<grid, 256, 0, ctx->stream>>>(n, vl, out); break;
        JUES_LINCOMB(1) JUES_LINCOMB(2) JUES_LINCOMB(3) JUES_LINCOMB(4) JUES_LINCOMB(5) JUES_LINCOMB(6)
        JUES_LINCOMB(7) JUES_LINCOMB(8) JUES_LINCOMB(9) JUES_LINCOMB(10) JUES_LINCOMB(11) JUES_LINCOMB(12)
        JUES_LINCOMB(13) JUES_LINCOMB(14) JUES_LINCOMB(15) JUES_LINCOMB(16)
#undef JUES_LINCOMB
    }
    JUES_CHECK_CUDA(cudaGetLastError());
}

}  // namespace jues
