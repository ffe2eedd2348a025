// Compressible Euler on the device-resident tree: EulerPhysics<DIM>
// (include/solver/EulerPhysics.hpp:17-170) advanced by amr_solver's forward
// Euler step (amr_solver.hpp:265-413) with the Rusanov flux.
//
// Built with -fmad=false: every product and sum rounds on its own, in the
// order the reference's C++ evaluates it, and division and square root are
// the correctly rounded IEEE operations, so each cell's result equals the
// reference CPU path's bit for bit.  What changes is how much is computed,
// never how: a face flux depends only on its two cells, so it is evaluated
// once per face (the reference evaluates it from both sides); the terms of a
// face flux that depend on one side only (the wave speed s_d = |u_d| + a and
// the physical flux m_k u_d + [k = d] p, u_d (E + p) of each direction d)
// depend only on the cell, so they are formed once, when the cell's value is
// written, and kept beside the state; and because correctly rounded
// division is monotonic, the minimum of dx_d / s over a patch's cells is
// dx_d / (maximum s), one division per patch and axis instead of one per
// cell.  Speeds are non-negative or NaN, so their comparisons and maxima
// are integer operations on the bit patterns (with the reference's NaN
// outcomes), which keeps them off the FP64 pipe, the bound of this kernel.
//
// One step is three launches: k_euler_finalize (step size from the previous
// minimum, clamped to the remaining time), k_euler_step (one block per tile
// of a patch: stage the tile and its face neighbours in shared memory, face
// fluxes, cell updates, side terms and the patch maximum of the new state),
// k_euler_halo (face ghosts of every field by the halo rules, and their side
// terms).
#include <algorithm>
#include <atomic>
#include <cfloat>

#include "amr_euler.cuh"

namespace amr_gb300 {
namespace {

constexpr unsigned long long kDblMaxBits = 0x7FEFFFFFFFFFFFFFull; // DBL_MAX
constexpr size_t             kEulerSmemLimit = 200 * 1024;

// Tile of a patch handled by one block: T[L] cells along layout dim L
// (dim 0 slowest), staged with one face-neighbour layer (box B = T + 2).
template <int R>
struct ETile {
    int    T[R], nt[R], B[R], bs[R], F[R], foff[R + 1];
    int    BC, TC, ntiles, threads;
    size_t smem;
};

template <int R>
constexpr int kNV = R + 2; // conservative fields
template <int R>
constexpr int kNP = R * (R + 2); // per direction d: s_d, m_k u_d + [k = d] p (k < R), u_d (E + p)
template <int R>
constexpr int kNQ = kNV<R> + kNP<R>; // staged quantities per cell

int largest_divisor_le(int n, int cap)
{
    for (int d = std::min(n, std::max(cap, 1)); d >= 1; --d)
        if (n % d == 0) return d;
    return 1;
}

template <int R>
bool pick_tile(const Geo& g, ETile<R>& t)
{
    for (int target : { 512, 256, 128, 64, 32, 16, 8, 4, 2, 1 }) {
        int left = target;
        for (int L = R - 1; L >= 0; --L) {
            t.T[L] = largest_divisor_le(g.n, left);
            left   = std::max(1, left / t.T[L]);
        }
        t.BC = t.TC = t.ntiles = 1;
        for (int L = 0; L < R; ++L) {
            t.nt[L] = g.n / t.T[L];
            t.B[L]  = t.T[L] + 2;
            t.BC *= t.B[L];
            t.TC *= t.T[L];
            t.ntiles *= t.nt[L];
        }
        int st = 1;
        for (int L = R - 1; L >= 0; --L) {
            t.bs[L] = st;
            st *= t.B[L];
        }
        t.foff[0] = 0;
        for (int L = 0; L < R; ++L) {
            int f = 1;
            for (int M = 0; M < R; ++M) f *= t.T[M] + (M == L ? 1 : 0);
            t.F[L]        = f;
            t.foff[L + 1] = t.foff[L] + f;
        }
        t.smem    = (static_cast<size_t>(kNQ<R>) * t.BC + static_cast<size_t>(kNV<R>) * t.foff[R]) * sizeof(double);
        t.threads = std::min(256, (t.TC + 31) / 32 * 32);
        if (t.smem <= kEulerSmemLimit) return true;
    }
    return false;
}

// The one-side terms of rusanovFlux (EulerPhysics.hpp:83-90, 113-127) and
// getMaxSpeed for every direction d, in the reference's operation order:
// q[d*(R+2)] = |u_d| + a, q[d*(R+2) + 1 + k] = m_k u_d (+ p when k = d),
// q[d*(R+2) + R + 1] = u_d (E + p).
template <int R>
__device__ __forceinline__ void side_terms(const double* U, double gamma, double* q)
{
    const double inv_rho = 1.0 / U[0];
    double       K       = 0.0;
#pragma unroll
    for (int d = 0; d < R; ++d) K += U[1 + d] * U[1 + d];
    K *= 0.5 * inv_rho;
    const double p  = (gamma - 1.0) * (U[R + 1] - K);
    const double a  = sqrt(gamma * p * inv_rho);
    const double Ep = U[R + 1] + p;
#pragma unroll
    for (int d = 0; d < R; ++d) {
        const double u = U[1 + d] * inv_rho;
        double*      o = q + d * (R + 2);
        o[0]           = fabs(u) + a;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            double f = U[1 + k] * u;
            if (k == d) f += p;
            o[1 + k] = f;
        }
        o[R + 1] = u * Ep;
    }
}

template <int R>
__device__ __forceinline__ void store_terms(double* prim, size_t fs, size_t at, const double* q)
{
#pragma unroll
    for (int j = 0; j < kNP<R>; ++j) prim[j * fs + at] = q[j];
}

// Wave speeds are |u| + a: +0 or positive, or NaN.  For such values the
// order of the bit patterns is the numeric order, so std::max(left, right)
// = (left < right) ? right : left is decided on the integers, NaN included
// (any comparison with NaN is false: the left value is kept).
__device__ __forceinline__ bool is_nan_bits(unsigned long long b) { return (b << 1) > (0x7FF0000000000000ull << 1); }

__device__ __forceinline__ double speed_max(double l, double r)
{
    const unsigned long long bl = static_cast<unsigned long long>(__double_as_longlong(l));
    const unsigned long long br = static_cast<unsigned long long>(__double_as_longlong(r));
    return (!is_nan_bits(bl) && !is_nan_bits(br) && bl < br) ? r : l;
}

// Running maximum of speeds as bit patterns; NaN speeds never count (they
// fail the reference's `speed > 1e-12`).
__device__ __forceinline__ unsigned long long speed_fold(unsigned long long m, double s)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(s));
    return (!is_nan_bits(b) && b > m) ? b : m;
}

// Rusanov flux across the face between staged cells cl (left) and cr
// (right) along Morton axis dir (EulerPhysics.hpp:102-128), from the states
// and the one-side terms of the two cells.
template <int R>
__device__ __forceinline__ void face_flux(const double* cq, int BC, int cl, int cr, int dir, double* F)
{
    constexpr int NV = kNV<R>;
    const int     q0 = (NV + dir * (R + 2)) * BC; // this direction's side terms
    const double  smax = speed_max(cq[q0 + cl], cq[q0 + cr]);
    F[0] = 0.5 * (cq[(1 + dir) * BC + cl] + cq[(1 + dir) * BC + cr] - smax * (cq[cr] - cq[cl]));
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const double mL = cq[(1 + k) * BC + cl], mR = cq[(1 + k) * BC + cr];
        F[1 + k] = 0.5 * (cq[q0 + (1 + k) * BC + cl] + cq[q0 + (1 + k) * BC + cr] - smax * (mR - mL));
    }
    const double EL = cq[(R + 1) * BC + cl], ER = cq[(R + 1) * BC + cr];
    F[R + 1] = 0.5 * (cq[q0 + (R + 1) * BC + cl] + cq[q0 + (R + 1) * BC + cr] - smax * (ER - EL));
}

// Block maximum of the per-thread speed maxima (bit patterns), then thread
// 0 folds dx_d / max into the global minimum (ordered bit patterns of
// non-negative doubles).  Speeds of at most 1e-12 never count
// (compute_time_step_cpu, amr_solver.hpp:384-397).
template <int R>
__device__ void fold_min_dt(unsigned long long* smax, const double* cs, unsigned long long* slot)
{
    __shared__ unsigned long long red[32][R];
#pragma unroll
    for (int d = 0; d < R; ++d) {
        unsigned long long v = smax[d];
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
            v                          = w > v ? w : v;
        }
        smax[d] = v;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
        for (int d = 0; d < R; ++d) red[warp][d] = smax[d];
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        double    m  = DBL_MAX;
#pragma unroll
        for (int d = 0; d < R; ++d) {
            unsigned long long b = red[0][d];
            for (int w = 1; w < nw; ++w) b = red[w][d] > b ? red[w][d] : b;
            const double S = __longlong_as_double(static_cast<long long>(b));
            if (S > 1e-12) {
                const double c = cs[d] / S;
                if (c < m) m = c;
            }
        }
        if (m < DBL_MAX) atomicMin(slot, static_cast<unsigned long long>(__double_as_longlong(m)));
    }
}

__global__ void k_euler_begin(unsigned long long* min_slot, int32_t* ctl, double* acc, double* rem, uint32_t* cnt,
                              double remaining)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    min_slot[0] = kDblMaxBits;
    min_slot[1] = kDblMaxBits;
    ctl[0]      = 0;
    ctl[1]      = 0;
    acc[0]      = 0.0;
    rem[0]      = remaining;
    cnt[0]      = 0;
}

// Side terms of the interior and face-ghost cells of every patch, and the
// minimum for the first step.  One block per patch.
template <int R>
__global__ void __launch_bounds__(256)
k_euler_prims(const double* __restrict__ state, double* __restrict__ prim, size_t fs, const int32_t* __restrict__ levels,
              int P, Geo g, double gamma, unsigned long long* min_slot)
{
    constexpr int NV = kNV<R>;
    const int     p  = blockIdx.x;
    if (p >= P) return; // uniform per block
    const size_t       pb = static_cast<size_t>(p) * g.flat;
    unsigned long long smax[R];
#pragma unroll
    for (int d = 0; d < R; ++d) smax[d] = 0ull;
    for (int c = threadIdx.x; c < g.flat; c += blockDim.x) {
        int outside = 0, rem = c;
#pragma unroll
        for (int L = R - 1; L >= 0; --L) {
            const int i = rem % g.P1;
            rem /= g.P1;
            outside += (i < g.h || i >= g.n + g.h) ? 1 : 0;
        }
        if (outside > 1) continue; // edge and corner ghosts: never read
        double U[NV], q[kNP<R>];
#pragma unroll
        for (int k = 0; k < NV; ++k) U[k] = state[k * fs + pb + c];
        side_terms<R>(U, gamma, q);
        store_terms<R>(prim, fs, pb + c, q);
        if (outside == 0)
#pragma unroll
            for (int d = 0; d < R; ++d) smax[d] = speed_fold(smax[d], q[d * (R + 2)]);
    }
    double cs[R];
#pragma unroll
    for (int d = 0; d < R; ++d) cs[d] = cell_size(g, d, levels[p]);
    fold_min_dt<R>(smax, cs, min_slot);
}

// Step size of the coming step (advance_batch_async's CPU loop,
// amr_solver.hpp:300-330): stop when no time is left or the clamped step is
// not positive; otherwise count the step.  Resets the other minimum slot,
// which the step fills.
__global__ void k_euler_finalize(unsigned long long* min_slot, int slot, double cfl, double* step_dt, int32_t* ctl,
                                 double* acc, double* rem, uint32_t* cnt)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    min_slot[slot ^ 1] = kDblMaxBits;
    ctl[0]             = 0;
    if (ctl[1]) return;
    const double remaining = rem[0];
    if (remaining <= 0.0) {
        ctl[1] = 1;
        return;
    }
    const double dt   = cfl * __longlong_as_double(static_cast<long long>(min_slot[slot]));
    const double step = dt < remaining ? dt : remaining;
    if (step <= 0.0) {
        ctl[1] = 1;
        return;
    }
    step_dt[0] = step;
    ctl[0]     = 1;
    acc[0]     = acc[0] + step;
    rem[0]     = remaining - step;
    cnt[0]     = cnt[0] + 1;
}

template <int R>
struct EulerStepArgs {
    Geo                 g;
    ETile<R>            t;
    const double*       in;
    double*             out;
    const double*       pin;
    double*             pout;
    size_t              fs;
    const int32_t*      levels;
    const double*       step_dt;
    const int32_t*      ctl;
    unsigned long long* next_min;
    double              gamma;
};

template <int R>
__device__ __forceinline__ int padded_of(const Geo& g, const int* o, const int* z)
{
    int li = 0;
#pragma unroll
    for (int L = 0; L < R; ++L) li += (o[L] + z[L] - 1 + g.h) * g.s[L];
    return li;
}

template <int R>
__global__ void __launch_bounds__(256) k_euler_step(EulerStepArgs<R> a)
{
    constexpr int   NV = kNV<R>, NQ = kNQ<R>;
    extern __shared__ double sm[];
    const ETile<R>& t  = a.t;
    const Geo&      g  = a.g;
    const int       p  = blockIdx.x / t.ntiles;
    int             rem = blockIdx.x - p * t.ntiles, o[R];
#pragma unroll
    for (int L = R - 1; L >= 0; --L) {
        o[L] = (rem % t.nt[L]) * t.T[L];
        rem /= t.nt[L];
    }
    const size_t  pb = static_cast<size_t>(p) * g.flat;
    const size_t  fs = a.fs;
    const double* in = a.in + pb;
    const double* pi = a.pin + pb;
    double*       out = a.out + pb;
    double*       po  = a.pout + pb;
    if (!a.ctl[0]) { // the advance has stopped: the state carries over
        for (int c = threadIdx.x; c < t.TC; c += blockDim.x) {
            int z[R], r = c;
#pragma unroll
            for (int L = R - 1; L >= 0; --L) {
                z[L] = r % t.T[L] + 1;
                r /= t.T[L];
            }
            const int li = padded_of<R>(g, o, z);
#pragma unroll
            for (int k = 0; k < NV; ++k) out[k * fs + li] = in[k * fs + li];
#pragma unroll
            for (int q = 0; q < kNP<R>; ++q) po[q * fs + li] = pi[q * fs + li];
        }
        return;
    }
    double* cq = sm;                  // NQ x BC staged cells
    double* fq = sm + NQ * t.BC;      // NV x FT face fluxes
    const int FT = t.foff[R];
    // stage the tile and its face neighbours
    for (int c = threadIdx.x; c < t.BC; c += blockDim.x) {
        int z[R], r = c, outside = 0;
#pragma unroll
        for (int L = R - 1; L >= 0; --L) {
            z[L] = r % t.B[L];
            r /= t.B[L];
            outside += (z[L] == 0 || z[L] == t.B[L] - 1) ? 1 : 0;
        }
        if (outside > 1) continue;
        const int li = padded_of<R>(g, o, z);
#pragma unroll
        for (int k = 0; k < NV; ++k) cq[k * t.BC + c] = in[k * fs + li];
#pragma unroll
        for (int q = 0; q < kNP<R>; ++q) cq[(NV + q) * t.BC + c] = pi[q * fs + li];
    }
    __syncthreads();
    // face fluxes, each face once
    for (int f = threadIdx.x; f < FT; f += blockDim.x) {
        int L = 0;
#pragma unroll
        for (int M = 1; M < R; ++M) L += f >= t.foff[M] ? 1 : 0;
        int r = f - t.foff[L], cl = 0;
#pragma unroll
        for (int M = R - 1; M >= 0; --M) {
            const int e  = t.T[M] + (M == L ? 1 : 0);
            const int fz = r % e;
            r /= e;
            cl += (M == L ? fz : fz + 1) * t.bs[M];
        }
        double F[NV];
        face_flux<R>(cq, t.BC, cl, cl + t.bs[L], R - 1 - L, F);
#pragma unroll
        for (int k = 0; k < NV; ++k) fq[k * FT + f] = F[k];
    }
    __syncthreads();
    const int          level = a.levels[p];
    const double       dt    = a.step_dt[0];
    double             cs[R], dt_over_dx[R];
    unsigned long long smax[R];
#pragma unroll
    for (int d = 0; d < R; ++d) {
        cs[d]         = cell_size(g, d, level);
        dt_over_dx[d] = dt / cs[d]; // the same for every cell of the patch
        smax[d]       = 0ull;
    }
    // cell updates: total -= dt/dx_d (F_right - F_left) over d = 0..rank-1
    for (int c = threadIdx.x; c < t.TC; c += blockDim.x) {
        int z[R], r = c;
#pragma unroll
        for (int L = R - 1; L >= 0; --L) {
            z[L] = r % t.T[L];
            r /= t.T[L];
        }
        double total[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) total[k] = 0.0;
#pragma unroll
        for (int d = 0; d < R; ++d) {
            const int L = R - 1 - d;
            int       fi = 0, st = 1;
#pragma unroll
            for (int M = R - 1; M >= 0; --M) {
                fi += z[M] * st;
                st *= t.T[M] + (M == L ? 1 : 0);
            }
            int sL = 1; // stride of dim L among this dim's faces
#pragma unroll
            for (int M = R - 1; M > L; --M) sL *= t.T[M];
            const int left = t.foff[L] + fi, right = left + sL;
#pragma unroll
            for (int k = 0; k < NV; ++k) total[k] -= dt_over_dx[d] * (fq[k * FT + right] - fq[k * FT + left]);
        }
        int bc = 0;
#pragma unroll
        for (int L = 0; L < R; ++L) bc += (z[L] + 1) * t.bs[L];
        double U[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) U[k] = cq[k * t.BC + bc] + total[k];
#pragma unroll
        for (int L = 0; L < R; ++L) ++z[L];
        const int li = padded_of<R>(g, o, z);
#pragma unroll
        for (int k = 0; k < NV; ++k) out[k * fs + li] = U[k];
        double q[kNP<R>];
        side_terms<R>(U, a.gamma, q);
        store_terms<R>(po, fs, li, q);
#pragma unroll
        for (int d = 0; d < R; ++d) smax[d] = speed_fold(smax[d], q[d * (R + 2)]);
    }
    fold_min_dt<R>(smax, cs, a.next_min);
}

// Face halo of every field (the same rules and arithmetic as the one-field
// exchange), then the side terms of the ghost layer next to the interior.
template <int R>
__global__ void __launch_bounds__(256)
k_euler_halo(double* __restrict__ buf, double* __restrict__ prim, size_t fs, const amr_halo_meta* __restrict__ meta,
             long long total, Geo g, double gamma)
{
    constexpr int   NV        = kNV<R>;
    const long long per_dir   = static_cast<long long>(g.h) * (g.cells / g.n);
    const long long per_patch = per_dir * g.ndir;
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long p = t / per_patch;
        const long long r = t - p * per_patch;
        const int       d = static_cast<int>(r / per_dir);
        int             f = static_cast<int>(r - d * per_dir);
        const int       L = d / 2, pos = d % 2;
        int             G[3] = { 0, 0, 0 };
        for (int k = R - 1; k >= 0; --k) {
            if (k == L) continue;
            G[k] = f % g.n + g.h;
            f /= g.n;
        }
        G[L]                  = pos ? g.n + g.h + f : f;
        const amr_halo_meta m = meta[p * g.ndir + d];
        const size_t        at = static_cast<size_t>(p) * g.flat + padded_index(g, G);
        double              U[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double* bk = buf + k * fs;
            if (m.relation == REL_NONE) {
                U[k] = bk[at];
            } else {
                U[k]   = ghost_value<double>(bk, g.flat, m, G, L, pos, g, bk + static_cast<size_t>(p) * g.flat);
                bk[at] = U[k];
            }
        }
        if (G[L] == (pos ? g.n + g.h : g.h - 1)) {
            double q[kNP<R>];
            side_terms<R>(U, gamma, q);
            store_terms<R>(prim, fs, at, q);
        }
    }
}

template <int R>
cudaError_t step_r(const EulerBufs& b, int cur, int slot, double gamma, double cfl, uint64_t* launches,
                   cudaEvent_t ev0, cudaEvent_t ev1)
{
    ETile<R> t{};
    if (!pick_tile<R>(b.g, t)) return cudaErrorInvalidValue;
    static std::atomic<uint64_t> smem_set{ 0 }; // devices whose limit is raised
    int                          dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(smem_set.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(k_euler_step<R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(kEulerSmemLimit));
        if (e != cudaSuccess) return e;
        smem_set.fetch_or(bit);
    }
    k_euler_finalize<<<1, 32, 0, b.stream>>>(b.min_slot, slot, cfl, b.step_dt, b.ctl, b.acc, b.rem, b.cnt);
    EulerStepArgs<R> a{};
    a.g        = b.g;
    a.t        = t;
    a.in       = b.state[cur];
    a.out      = b.state[cur ^ 1];
    a.pin      = b.prim[cur];
    a.pout     = b.prim[cur ^ 1];
    a.fs       = b.fstride;
    a.levels   = b.levels;
    a.step_dt  = b.step_dt;
    a.ctl      = b.ctl;
    a.next_min = b.min_slot + (slot ^ 1);
    a.gamma    = gamma;
    if (ev0) cudaEventRecord(ev0, b.stream);
    if (b.P > 0)
        k_euler_step<R><<<static_cast<unsigned>(b.P) * t.ntiles, t.threads, t.smem, b.stream>>>(a);
    if (ev1) cudaEventRecord(ev1, b.stream);
    const long long total = static_cast<long long>(b.P) * b.g.ndir * b.g.h * (b.g.cells / b.g.n);
    if (total > 0) {
        const unsigned grid = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 152LL * 64));
        k_euler_halo<R><<<grid, 256, 0, b.stream>>>(b.state[cur ^ 1], b.prim[cur ^ 1], b.fstride, b.meta, total, b.g,
                                                    gamma);
    }
    *launches += 1 + (b.P > 0 ? 1 : 0) + (total > 0 ? 1 : 0);
    return cudaGetLastError();
}

template <int R>
cudaError_t begin_r(const EulerBufs& b, int cur, double gamma, double remaining, uint64_t* launches)
{
    k_euler_begin<<<1, 32, 0, b.stream>>>(b.min_slot, b.ctl, b.acc, b.rem, b.cnt, remaining);
    if (b.P > 0)
        k_euler_prims<R><<<b.P, 256, 0, b.stream>>>(b.state[cur], b.prim[cur], b.fstride, b.levels, b.P, b.g, gamma,
                                                    b.min_slot);
    *launches += 1 + (b.P > 0 ? 1 : 0);
    return cudaGetLastError();
}

} // namespace

cudaError_t euler_begin(const EulerBufs& b, int cur, double gamma, double remaining, uint64_t* launches)
{
    return b.g.rank == 2 ? begin_r<2>(b, cur, gamma, remaining, launches)
                         : begin_r<3>(b, cur, gamma, remaining, launches);
}

cudaError_t euler_step(const EulerBufs& b, int cur, int slot, double gamma, double cfl, uint64_t* launches,
                       cudaEvent_t ev0, cudaEvent_t ev1)
{
    return b.g.rank == 2 ? step_r<2>(b, cur, slot, gamma, cfl, launches, ev0, ev1)
                         : step_r<3>(b, cur, slot, gamma, cfl, launches, ev0, ev1);
}

bool euler_supported(const Geo& g)
{
    if (g.rank == 2) {
        ETile<2> t{};
        return pick_tile<2>(g, t);
    }
    ETile<3> t{};
    return pick_tile<3>(g, t);
}

} // namespace amr_gb300
