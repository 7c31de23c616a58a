// CMFD on the pin mesh (cmfd.cpp:171-666): surface coupling coefficients,
// the 5-point operator per group, then the CMFD power iteration with one
// preconditioned BiCGSTAB solve per group.
//
// One CTA runs a whole CMFD solve (cmfd_body: every solve of a batch, and
// single solves up to 1024 cells). Tiny meshes (up to 64 cells) run on a
// single warp, so every reduction is a shuffle tree and every barrier a warp
// barrier; larger meshes use 4 to 16 warps with one block barrier per
// reduction. Work vectors live in shared memory when they fit. A single
// solve of a larger mesh runs on a thread-block cluster instead
// (cmfd_body_cluster, below).
#include <algorithm>
#include <mutex>
#include <string>

#include "kernels.cuh"

namespace mocgpu {

namespace {

// Warp sum of two doubles with five FP64 adds per lane instead of ten: after
// one exchange the even lanes carry a and the odd lanes b, then a butterfly
// over the remaining bits sums each; every lane ends with both totals.
__device__ __forceinline__ void warp_sum2(double &a, double &b)
{
    const unsigned full = 0xffffffffu;
    const bool odd = threadIdx.x & 1;
    double keep = odd ? b : a;
    const double send = odd ? a : b;
    keep += __shfl_xor_sync(full, send, 1);
#pragma unroll
    for (int o = 2; o < 32; o <<= 1) keep += __shfl_xor_sync(full, keep, o);
    const double other = __shfl_xor_sync(full, keep, 1);
    a = odd ? other : keep;
    b = odd ? keep : other;
}

// Shared doubles a CTA of nw warps needs for gathered block sums: every
// lane's two partials and the two totals.
__host__ __device__ constexpr int gather_scratch(int nw) { return 64 * nw + 8; }

struct Blk {
    int nw; // warps in the CTA
    double *scratch;
    int buf = 0;
    // Gathered sums (scratch of gather_scratch(nw) doubles): every lane
    // stores its partial, one warp adds them up and publishes the total, at
    // two barriers per sum instead of one. The FP64 pipe of an SM takes 16
    // cycles per warp instruction, and a shuffle tree in every warp spends
    // nw times the FP64 instructions of one warp summing the lanes' column
    // sums: with four warps that was about 40 % of a BiCGSTAB iteration's
    // FP64 work.
    bool gather = false;
    __device__ void sync() const
    {
        if (nw == 1) __syncwarp();
        else __syncthreads();
    }
    // The FP64 adds of a gathered sum run on the warp that gathers it. Warp
    // w issues from scheduler w % 4, and with five warps scheduler 0 also
    // carries warp 4's rows, so the sums are gathered by warps 1-3 (sum2:
    // one value each on warps 2 and 3, sum: warp 1), spreading their FP64
    // instructions over the less loaded schedulers' pipes.
    __device__ int gather_warp(int k) const { return nw > 3 ? 1 + k : (nw > 1 ? k % nw : 0); }
    __device__ double gather_one(const double *p) const
    {
        const int lane = threadIdx.x & 31;
        double x = p[lane];
        for (int w = 1; w < nw; w++) x += p[lane + 32 * w];
        return warp_sum(x);
    }
    __device__ void gathered2(double &a, double &b)
    {
        double *pa = scratch, *pb = scratch + 32 * nw, *res = scratch + 64 * nw;
        pa[threadIdx.x] = a;
        pb[threadIdx.x] = b;
        __syncthreads();
        const int w = threadIdx.x >> 5;
        if (w == gather_warp(1)) {
            const double x = gather_one(pa);
            if ((threadIdx.x & 31) == 0) res[0] = x;
        }
        if (w == gather_warp(2)) {
            const double y = gather_one(pb);
            if ((threadIdx.x & 31) == 0) res[1] = y;
        }
        __syncthreads();
        a = res[0];
        b = res[1];
    }
    __device__ double gathered(double a)
    {
        double *pa = scratch, *res = scratch + 64 * nw;
        pa[threadIdx.x] = a;
        __syncthreads();
        if ((threadIdx.x >> 5) == gather_warp(0)) {
            const double x = gather_one(pa);
            if ((threadIdx.x & 31) == 0) res[0] = x;
        }
        __syncthreads();
        return res[0];
    }
    // Two block sums with a single barrier (double-buffered scratch); the
    // per-warp partials are combined pairwise so the adds form a tree.
    __device__ void sum2(double &a, double &b)
    {
        if (gather && nw > 1) return gathered2(a, b);
        warp_sum2(a, b);
        if (nw == 1) return;
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        double *s = scratch + buf * 64;
        if (lane == 0) {
            s[wid] = a;
            s[32 + wid] = b;
        }
        __syncthreads();
        a = tree(s, nw);
        b = tree(s + 32, nw);
        buf ^= 1;
    }
    // One block sum (five FP64 adds per lane in the warp stage).
    __device__ double sum(double a)
    {
        if (gather && nw > 1) return gathered(a);
        a = warp_sum(a);
        if (nw == 1) return a;
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        double *s = scratch + buf * 64;
        if (lane == 0) s[wid] = a;
        __syncthreads();
        a = tree(s, nw);
        buf ^= 1;
        return a;
    }
    // sum of v[0..n) as a pairwise tree (same order in every thread)
    __device__ static double tree(const double *v, int n)
    {
        if (n == 4) return (v[0] + v[1]) + (v[2] + v[3]);
        double t = 0.0;
        for (int w = 0; w < n; w++) t += v[w];
        return t;
    }
};

__device__ __forceinline__ int cell_of(const CmfdView &c, int ix, int iy) { return iy * c.nx + ix; }

__device__ int coarse_surf(const CmfdView &c, int cell, int s)
{
    const int nx = c.nx, ny = c.ny;
    int ix = cell % nx, iy = cell / nx;
    int nxy = (nx + 1) * ny + (ny + 1) * nx;
    switch (s) {
    case EAST: return (nx + 1) * iy + ix + 1 + nx * ny;
    case WEST: return (nx + 1) * iy + ix + nx * ny;
    case NORTH: return nx * ny + (nx + 1) * ny + (ny + 1) * ix + iy + 1;
    case SOUTH: return (nx + 1) * ny + (ny + 1) * ix + iy + nx * ny;
    case BOTTOM: return nx * iy + ix;
    default: return nx * ny + nxy + nx * iy + ix; // TOP
    }
}
__device__ int neighbor(const CmfdView &c, int cell, int s)
{
    int ix = cell % c.nx, iy = cell / c.nx;
    switch (s) {
    case NORTH: return iy < c.ny - 1 ? cell + c.nx : -1;
    case SOUTH: return iy > 0 ? cell - c.nx : -1;
    case EAST: return ix < c.nx - 1 ? cell + 1 : -1;
    case WEST: return ix > 0 ? cell - 1 : -1;
    default: return -1;
    }
}
__device__ double area(const CmfdView &c, int cell, int s)
{
    int ix = cell % c.nx, iy = cell / c.nx;
    if (s == EAST || s == WEST) return c.dy[iy] * c.hz;
    if (s == NORTH || s == SOUTH) return c.dx[ix] * c.hz;
    return c.dx[ix] * c.dy[iy];
}
__device__ void surf_info(const CmfdView &c, int surf, int &c1, int &c2, int &nrm)
{
    const int nx = c.nx, ny = c.ny;
    int nsz = nx * ny + (nx + 1) * ny + (ny + 1) * nx;
    int s = surf % nsz;
    int iz = surf / nsz;
    if (s < nx * ny) {
        nrm = Z_NORM;
        c1 = (iz > 0) ? s : -1;
        c2 = (iz < 1) ? s : -1;
    } else if (s < nx * ny + (nx + 1) * ny) {
        nrm = X_NORM;
        int t = s - nx * ny;
        int iy = t / (nx + 1), ix = t % (nx + 1);
        c1 = ix > 0 ? cell_of(c, ix - 1, iy) : -1;
        c2 = ix < nx ? cell_of(c, ix, iy) : -1;
    } else {
        nrm = Y_NORM;
        int t = s - nx * ny - (nx + 1) * ny;
        int iy = t % (ny + 1), ix = t / (ny + 1);
        c1 = iy > 0 ? cell_of(c, ix, iy - 1) : -1;
        c2 = iy < ny ? cell_of(c, ix, iy) : -1;
    }
}
__device__ double thickness(const CmfdView &c, int cell, int nrm)
{
    if (nrm == X_NORM) return c.dx[cell % c.nx];
    if (nrm == Y_NORM) return c.dy[cell / c.nx];
    return c.hz;
}
__device__ __forceinline__ double cell_vol(const CmfdView &c, int i) { return c.dx[i % c.nx] * c.dy[i / c.nx] * c.hz; }

// The operator of each group is kept column-scaled by the Jacobi
// preconditioner: m[0..n) holds the diagonal d (1 where it vanishes), m[5n..6n)
// its inverse, and m[n..5n) the off-diagonal entries A_ij / d_j of the west,
// east, south and north neighbours. Right-preconditioned BiCGSTAB applies
// A D^-1 to its search vectors, which is this operator with a unit diagonal:
// four FP64 multiply-adds per row and no separate preconditioner product.

// Row i of A D^-1 applied to x (unit diagonal).
__device__ __forceinline__ double spmv_row(const double *__restrict__ m, const double *x, int i, int n, int nx)
{
    double v = x[i];
    int ix = i % nx;
    if (ix > 0) v += m[n + i] * x[i - 1];
    if (ix < nx - 1) v += m[2 * n + i] * x[i + 1];
    if (i >= nx) v += m[3 * n + i] * x[i - nx];
    if (i + nx < n) v += m[4 * n + i] * x[i + nx];
    return v;
}

// b_g = (chi_g fs + sum_{g'!=g} S(g<-g') phi_g') V
// sum over gg != skip of a[gg * sa] * b[gg * sb] in order of gg, with the
// loads of eight groups issued together (the CMFD CTA is latency-bound:
// a loop of dependent load-multiply-adds waits out one memory latency per
// group)
__device__ __forceinline__ double group_dot(const double *a, int sa, const double *b, int sb, int G, int skip)
{
    double s = 0.0;
    for (int g0 = 0; g0 < G; g0 += 8) {
        double x[8], y[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int gg = g0 + j;
            const bool ok = gg < G && gg != skip;
            x[j] = ok ? a[(size_t)gg * sa] : 0.0;
            y[j] = ok ? b[(size_t)gg * sb] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < 8; j++) s += x[j] * y[j];
    }
    return s;
}

__device__ void build_source(const CmfdView &c, int g, double *b)
{
    const int n = c.n_cell, G = c.G;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double s = c.xsch[(size_t)i * G + g] * c.fs[i];
        s += group_dot(c.scat + ((size_t)i * G + g) * G, 1, c.flux + i, n, G, g);
        b[i] = s * cell_vol(c, i);
    }
}

// Preconditioned BiCGSTAB (van der Vorst 1992) with a diagonal (Jacobi)
// preconditioner applied from the right, as Eigen's BiCGSTAB with its
// DiagonalPreconditioner (the solver of cmfd.cpp), stopping on the true
// residual, ||r||^2 <= tol^2 ||b||^2, or after max_it iterations, and
// restarting the shadow residual when it becomes orthogonal. The iteration
// runs on xh = D x with the column-scaled operator (xh += alpha p + omega s
// is x += alpha D^-1 p + omega D^-1 s), which gives the same iterates as
// applying D^-1 to p and s. x is in/out; w holds 8 work vectors; rr0 returns
// ||b - A x||^2 of the incoming x.
// The same iteration with each thread's R rows of every vector in registers
// (rows i = threadIdx.x + j blockDim.x): only the two vectors the operator
// is applied to, p and s, go through shared memory (w and w + n), where the
// neighbours' entries are read. Each row's off-diagonal entries are loaded
// once per solve; a missing neighbour has a zero entry and reads a slot in
// range (the index clamped), which adds exactly nothing. The arithmetic of every entry, the
// block sums and the barriers are those of the shared-memory form below:
// the shared-memory traffic of an iteration drops from about 35 accesses
// per row to 10.
template <int R>
__device__ int bicgstab_reg(const CmfdView &c, Blk &B, const double *m, const double *b, double *x, double tol,
                            int max_it, double *w, double &rr0)
{
    const int n = c.n_cell, nx = c.nx, bd = blockDim.x;
    double *P = w, *S = w + n;
    double xr[R], rr_[R], r0[R], p[R], v[R], bv[R], cw[R], ce[R], cs[R], cn[R];
    bool ok[R];
#pragma unroll
    for (int j = 0; j < R; j++) {
        const int i = threadIdx.x + j * bd;
        ok[j] = i < n;
        const int ii = ok[j] ? i : 0;
        const int ix = ii % nx;
        cw[j] = (ok[j] && ix > 0) ? m[n + ii] : 0.0;
        ce[j] = (ok[j] && ix < nx - 1) ? m[2 * n + ii] : 0.0;
        cs[j] = (ok[j] && ii >= nx) ? m[3 * n + ii] : 0.0;
        cn[j] = (ok[j] && ii + nx < n) ? m[4 * n + ii] : 0.0;
        bv[j] = ok[j] ? b[ii] : 0.0;
        xr[j] = ok[j] ? x[ii] * m[ii] : 0.0;
        p[j] = 0.0;
        v[j] = 0.0;
    }
    // row j of the unit-diagonal operator applied to the vector in V (own entry e)
    auto apply = [&](const double *V, int j, double e) {
        const int i = threadIdx.x + j * bd;
        double a = e;
        a = fma(cw[j], V[max(i - 1, 0)], a);
        a = fma(ce[j], V[min(i + 1, n - 1)], a);
        a = fma(cs[j], V[max(i - nx, 0)], a);
        a = fma(cn[j], V[min(i + nx, n - 1)], a);
        return a;
    };
    // r = b - A xh, with xh published in x
    auto residual = [&](double &acc) {
#pragma unroll
        for (int j = 0; j < R; j++)
            if (ok[j]) x[threadIdx.x + j * bd] = xr[j];
        B.sync();
#pragma unroll
        for (int j = 0; j < R; j++) {
            const double ri = ok[j] ? bv[j] - apply(x, j, xr[j]) : 0.0;
            rr_[j] = ri;
            r0[j] = ri;
            acc += ri * ri;
        }
    };
    const double eps2 = 2.220446049250313e-16 * 2.220446049250313e-16;
    double rr = 0.0, bb = 0.0;
    residual(rr);
#pragma unroll
    for (int j = 0; j < R; j++) bb += bv[j] * bv[j];
    B.sum2(rr, bb);
    rr0 = rr;
    if (bb == 0.0) {
#pragma unroll
        for (int j = 0; j < R; j++)
            if (ok[j]) x[threadIdx.x + j * bd] = 0.0;
        B.sync();
        return 0;
    }
    double r0_sq = rr, rho = 1.0, alpha = 1.0, om = 1.0;
    const double tol2 = tol * tol * bb;
    int it = 0, restarts = 0;
    double rho_new = rr;
    while (rr > tol2 && it < max_it) {
        double rho_old = rho;
        rho = rho_new;
        if (fabs(rho) < eps2 * r0_sq) {
            B.sync();
            double acc = 0.0;
            residual(acc);
            acc = B.sum(acc);
            rho = r0_sq = acc;
            if (restarts++ == 0) it = 0;
        }
        // Eigen's (rho / rho_old) (alpha / omega) with one division
        const double beta = (rho * alpha) / (rho_old * om);
#pragma unroll
        for (int j = 0; j < R; j++) {
            p[j] = rr_[j] + beta * (p[j] - om * v[j]);
            if (ok[j]) P[threadIdx.x + j * bd] = p[j];
        }
        B.sync();
        double r0v = 0.0;
#pragma unroll
        for (int j = 0; j < R; j++) {
            v[j] = ok[j] ? apply(P, j, p[j]) : 0.0;
            r0v += r0[j] * v[j];
        }
        r0v = B.sum(r0v);
        alpha = rho / r0v;
        double sv[R];
#pragma unroll
        for (int j = 0; j < R; j++) {
            sv[j] = rr_[j] - alpha * v[j];
            if (ok[j]) S[threadIdx.x + j * bd] = sv[j];
        }
        B.sync();
        double tt = 0.0, ts = 0.0, tv[R];
#pragma unroll
        for (int j = 0; j < R; j++) {
            tv[j] = ok[j] ? apply(S, j, sv[j]) : 0.0;
            tt += tv[j] * tv[j];
            ts += tv[j] * sv[j];
        }
        B.sum2(tt, ts);
        om = (tt > 0.0) ? ts / tt : 0.0;
        double nrr = 0.0, nrho = 0.0;
#pragma unroll
        for (int j = 0; j < R; j++) {
            xr[j] += alpha * p[j] + om * sv[j];
            const double ri = sv[j] - om * tv[j];
            rr_[j] = ri;
            nrr += ri * ri;
            nrho += r0[j] * ri;
        }
        B.sum2(nrr, nrho);
        rr = nrr;
        rho_new = nrho;
        it++;
    }
    B.sync();
#pragma unroll
    for (int j = 0; j < R; j++)
        if (ok[j]) x[threadIdx.x + j * bd] = xr[j] * m[5 * n + threadIdx.x + j * bd];
    B.sync();
    return it;
}

__device__ int bicgstab(const CmfdView &c, Blk &B, const double *m, const double *b, double *x, double tol, int max_it,
                        double *w, double &rr0)
{
    const int n = c.n_cell, nx = c.nx;
    switch ((n + (int)blockDim.x - 1) / (int)blockDim.x) {
    case 1: return bicgstab_reg<1>(c, B, m, b, x, tol, max_it, w, rr0);
    case 2: return bicgstab_reg<2>(c, B, m, b, x, tol, max_it, w, rr0);
    default: break;
    }
    double *r = w, *r0 = w + n, *p = w + 2 * n, *v = w + 3 * n, *s = w + 6 * n, *t = w + 7 * n;
    const double eps2 = 2.220446049250313e-16 * 2.220446049250313e-16;
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] *= m[i];
    B.sync();
    double rr = 0.0, bb = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double ri = b[i] - spmv_row(m, x, i, n, nx);
        r[i] = ri;
        r0[i] = ri;
        p[i] = 0.0;
        v[i] = 0.0;
        rr += ri * ri;
        bb += b[i] * b[i];
    }
    B.sum2(rr, bb);
    rr0 = rr;
    if (bb == 0.0) {
        for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = 0.0;
        B.sync();
        return 0;
    }
    double r0_sq = rr, rho = 1.0, alpha = 1.0, om = 1.0;
    const double tol2 = tol * tol * bb;
    int it = 0, restarts = 0;
    double rho_new = rr;
    while (rr > tol2 && it < max_it) {
        double rho_old = rho;
        rho = rho_new;
        if (fabs(rho) < eps2 * r0_sq) {
            B.sync();
            double acc = 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                double ri = b[i] - spmv_row(m, x, i, n, nx);
                r[i] = ri;
                r0[i] = ri;
                acc += ri * ri;
            }
            acc = B.sum(acc);
            rho = r0_sq = acc;
            if (restarts++ == 0) it = 0;
        }
        // Eigen's (rho / rho_old) (alpha / omega) with one division
        const double beta = (rho * alpha) / (rho_old * om);
        for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = r[i] + beta * (p[i] - om * v[i]);
        B.sync();
        double r0v = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double vi = spmv_row(m, p, i, n, nx);
            v[i] = vi;
            r0v += r0[i] * vi;
        }
        r0v = B.sum(r0v);
        alpha = rho / r0v;
        for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = r[i] - alpha * v[i];
        B.sync();
        double tt = 0.0, ts = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double ti = spmv_row(m, s, i, n, nx);
            t[i] = ti;
            tt += ti * ti;
            ts += ti * s[i];
        }
        B.sum2(tt, ts);
        om = (tt > 0.0) ? ts / tt : 0.0;
        double nrr = 0.0, nrho = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            x[i] += alpha * p[i] + om * s[i];
            double ri = s[i] - om * t[i];
            r[i] = ri;
            nrr += ri * ri;
            nrho += r0[i] * ri;
        }
        B.sum2(nrr, nrho);
        rr = nrr;
        rho_new = nrho;
        it++;
    }
    B.sync();
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] *= m[5 * n + i];
    B.sync();
    return it;
}

__device__ void fission_source(const CmfdView &c, double k)
{
    const int n = c.n_cell, G = c.G;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        c.fs[i] = group_dot(c.xsnf + (size_t)i * G, 1, c.flux + i, n, G, -1) * (1.0 / k);
}

__device__ double total_fission(const CmfdView &c, Blk &B)
{
    const int n = c.n_cell, G = c.G;
    double f = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) f += group_dot(c.xsnf + (size_t)i * G, 1, c.flux + i, n, G, -1);
    return B.sum(f);
}

// ||M_g x - b_g||^2 with x the group flux (A_ij = m_ij d_j off the diagonal)
__device__ double residual_g(const CmfdView &c, Blk &B, const double *m, const double *x, const double *b)
{
    const int n = c.n_cell, nx = c.nx;
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double v = m[i] * x[i];
        int ix = i % nx;
        if (ix > 0) v += m[n + i] * (m[i - 1] * x[i - 1]);
        if (ix < nx - 1) v += m[2 * n + i] * (m[i + 1] * x[i + 1]);
        if (i >= nx) v += m[3 * n + i] * (m[i - nx] * x[i - nx]);
        if (i + nx < n) v += m[4 * n + i] * (m[i + nx] * x[i + nx]);
        double d = v - b[i];
        acc += d * d;
    }
    return B.sum(acc);
}

} // namespace

__device__ void cmfd_body(CmfdView c, int vec_in_smem)
{
    extern __shared__ __align__(16) double sm[];
    Blk B;
    B.nw = blockDim.x >> 5;
    B.scratch = sm; // gather_scratch(nw) doubles
    B.gather = true;
    const int sc = gather_scratch(B.nw);
    const int n = c.n_cell, G = c.G, ns = c.n_surf;
    // work vectors: b, x (group flux copy), 8 BiCGSTAB vectors
    double *vec = vec_in_smem ? sm + sc : c.vec;
    // mode 2: the current group's operator is also staged in shared memory;
    // mode 3: every group's operator, staged once after it is built
    double *ms = (vec_in_smem >= 2) ? sm + sc + 10 * n : nullptr;
    double *b = vec, *x = vec + n, *w = vec + 2 * n;
    double k = *c.k;
    if (c.fixup)
        for (int i = threadIdx.x; i < n * G; i += blockDim.x) c.flux[i] = fmax(c.flux[i], 0.0);
    B.sync();

    // surface coupling coefficients (cmfd.cpp:404-499)
    for (int idx = threadIdx.x; idx < G * ns; idx += blockDim.x) {
        int g = idx / ns, is = idx % ns;
        int c1, c2, nrm;
        surf_info(c, is, c1, c2, nrm);
        int lo_bc = (nrm == X_NORM) ? c.bc[WEST] : (nrm == Y_NORM) ? c.bc[SOUTH] : c.bc[BOTTOM];
        int hi_bc = (nrm == X_NORM) ? c.bc[EAST] : (nrm == Y_NORM) ? c.bc[NORTH] : c.bc[TOP];
        double d1 = (c1 > -1) ? (1.0 / (3.0 * c.xstr[(size_t)c1 * G + g])) / thickness(c, c1, nrm)
                              : (lo_bc == (int)BoundaryType::VACUUM ? 0.5 / 2.0 : 0.0);
        double d2 = (c2 > -1) ? (1.0 / (3.0 * c.xstr[(size_t)c2 * G + g])) / thickness(c, c2, nrm)
                              : (hi_bc == (int)BoundaryType::VACUUM ? 0.5 / 2.0 : 0.0);
        double dt = 2.0 * d1 * d2 / (d1 + d2);
        double stil = (d1 > 0.0) ? d1 / (d1 + d2) : d2 / (d1 + d2);
        double dh = 0.0, sh = 0.0;
        if (nrm != Z_NORM && c.has_radial) {
            double j = c.cur[(size_t)g * ns + is];
            double sfc = c.sflux[(size_t)g * ns + is];
            double fl = c1 >= 0 ? c.flux[(size_t)g * n + c1] : 0.0;
            double fr = c2 >= 0 ? c.flux[(size_t)g * n + c2] : 0.0;
            dh = (j + dt * (fr - fl)) / (fl + fr);
            if (!isfinite(dh)) dh = 0.0;
            sh = (c1 >= 0) ? (sfc - stil * fl - (1.0 - stil) * fr) / (fl + fr) : (sfc - stil * fr) / fr;
        }
        c.d_tilde[idx] = dt;
        c.s_tilde[idx] = stil;
        c.d_hat[idx] = dh;
        c.s_hat[idx] = sh;
    }
    B.sync();
    // 5-point operator per group (cmfd.cpp:506-544)
    for (int idx = threadIdx.x; idx < G * n; idx += blockDim.x) {
        int g = idx / n, i = idx % n;
        const double *dt = c.d_tilde + (size_t)g * ns;
        const double *dh = c.d_hat + (size_t)g * ns;
        double diag = cell_vol(c, i) * c.xsrm[(size_t)i * G + g];
        const int surfs[6] = {EAST, NORTH, WEST, SOUTH, TOP, BOTTOM};
        for (int k6 = 0; k6 < 6; k6++) {
            int s = surfs[k6];
            int sf = coarse_surf(c, i, s);
            double h = dh[sf];
            if (s == WEST || s == SOUTH || s == BOTTOM) h = -h;
            diag += area(c, i, s) * (dt[sf] + h);
        }
        double *m = c.mat + (size_t)g * 6 * n;
        m[i] = (diag != 0.0) ? diag : 1.0;
        m[(size_t)5 * n + i] = (diag != 0.0) ? 1.0 / diag : 1.0; // Jacobi preconditioner
        const int offs[4] = {WEST, EAST, SOUTH, NORTH};
        for (int q = 0; q < 4; q++) {
            int s = offs[q];
            double v = 0.0;
            if (neighbor(c, i, s) >= 0) {
                int sf = coarse_surf(c, i, s);
                double h = dh[sf];
                if (s == WEST || s == SOUTH) h = -h;
                v = area(c, i, s) * (h - dt[sf]);
            }
            m[(size_t)(q + 1) * n + i] = v;
        }
    }
    B.sync();
    // column scaling by the neighbour's inverse diagonal
    for (int idx = threadIdx.x; idx < G * n; idx += blockDim.x) {
        const int g = idx / n, i = idx % n, ix = i % c.nx;
        double *m = c.mat + (size_t)g * 6 * n;
        const double *dinv = m + (size_t)5 * n;
        if (ix > 0) m[(size_t)n + i] *= dinv[i - 1];
        if (ix < c.nx - 1) m[(size_t)2 * n + i] *= dinv[i + 1];
        if (i >= c.nx) m[(size_t)3 * n + i] *= dinv[i - c.nx];
        if (i + c.nx < n) m[(size_t)4 * n + i] *= dinv[i + c.nx];
    }
    B.sync();
    if (vec_in_smem == 3)
        for (int i = threadIdx.x; i < 6 * n * G; i += blockDim.x) ms[i] = c.mat[i];

    fission_source(c, k);
    B.sync();
    double tfis = total_fission(c, B);
    double r0 = 0.0;
    for (int g = 0; g < G; g++) {
        build_source(c, g, b);
        B.sync();
        r0 += residual_g(c, B, c.mat + (size_t)g * 6 * n, c.flux + (size_t)g * n, b);
    }
    r0 = sqrt(r0) / (double)(n * G);
    const double tol = c.resid_reduction * r0;

    int iter = 0, bic_its = 0;
    double psi_err = 1.0, ri = 0.0, k_old = k;
    while (true) {
        iter++;
        for (int i = threadIdx.x; i < n; i += blockDim.x) c.fs_old[i] = c.fs[i];
        B.sync();
        fission_source(c, k);
        double tfis_old = tfis;
        ri = 0.0;
        for (int g = 0; g < G; g++) {
            const double *m = c.mat + (size_t)g * 6 * n;
            double *fg = c.flux + (size_t)g * n;
            B.sync();
            if (vec_in_smem == 3) {
                m = ms + (size_t)g * 6 * n;
            } else if (ms) {
                // 16-byte asynchronous copies, all in flight at once (a loop
                // of loads and stores waits out one memory latency per pass);
                // both arrays start 16-byte aligned and 6n doubles are whole
                // 16-byte chunks
                const int nc = 3 * n;
                for (int i = threadIdx.x; i < nc; i += blockDim.x) {
                    const unsigned d = (unsigned)__cvta_generic_to_shared(ms + 2 * i);
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(m + 2 * i) : "memory");
                }
                asm volatile("cp.async.commit_group;\n" ::: "memory");
                asm volatile("cp.async.wait_group 0;\n" ::: "memory");
                m = ms;
            }
            build_source(c, g, b);
            for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = fg[i];
            B.sync();
            double rr0 = 0.0;
            bic_its += bicgstab(c, B, m, b, x, tol, 150, w, rr0);
            ri += rr0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) fg[i] = x[i];
        }
        B.sync();
        ri = sqrt(ri) / (double)(n * G);
        tfis = total_fission(c, B);
        k_old = k;
        k = k * tfis / tfis_old;
        double pe = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double e = c.fs[i] - c.fs_old[i];
            pe += e * e;
        }
        psi_err = sqrt(B.sum(pe));
        if ((fabs(k - k_old) < c.k_tol && psi_err < c.psi_tol && ri / r0 < c.resid_reduction) || iter > c.max_iter)
            break;
    }
    for (int i = threadIdx.x; i < n * G; i += blockDim.x)
        if (c.flux[i] < 0.0) c.flux[i] = -c.flux[i];
    B.sync();
    if (threadIdx.x == 0) {
        *c.k = k;
        c.stats[0] = iter;
        c.stats[1] = r0;
        c.stats[2] = ri / r0;
        c.stats[3] = psi_err;
        c.stats[4] = bic_its;
        if (!isfinite(k)) atomicOr(c.status, (unsigned)DEV_NAN);
    }
}

// ---------------------------------------------------------------------------
// CMFD of one solve on a thread-block cluster: the CTAs of the cluster split
// the coarse cells into contiguous slices and each keeps its slice of every
// work vector and of the current group's operator in its shared memory. A
// matrix row whose neighbour lies in another CTA's slice reads it from that
// CTA's shared memory (distributed shared memory); every block sum is
// completed across the cluster by writing each CTA's total into every CTA's
// exchange slots and adding the slots in rank order after a cluster barrier,
// so all CTAs hold bit-identical sums and take the same branches at every
// loop test (the barriers of the cluster stay matched). Data one CTA writes to
// global memory for another (fixed-up fluxes, surface coefficients, inverse
// diagonals) is read back through L2 (ld.global.cg) after a cluster barrier.
// The FP64 work of a BiCGSTAB iteration is spread over several SMs' FP64
// pipes, which is what bounds the one-CTA solve of a single large mesh.
namespace {

__device__ __forceinline__ unsigned cl_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_nrank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;\n" : "=r"(r));
    return r;
}
// Barrier of all threads of the cluster (a warp may arrive diverged, after
// loops of uneven trip counts: it reconverges first).
__device__ __forceinline__ void cl_sync()
{
    __syncwarp();
    asm volatile("barrier.cluster.arrive.release;\n" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory");
}
// shared-memory address `p` (of this CTA's layout) in CTA `rank` of the cluster
__device__ __forceinline__ unsigned peer_addr(const void *p, unsigned rank)
{
    unsigned a = (unsigned)__cvta_generic_to_shared(p), r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ double ld_peer(const double *p, unsigned rank)
{
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];\n" : "=d"(v) : "r"(peer_addr(p, rank)) : "memory");
    return v;
}
__device__ __forceinline__ void st_peer(double *p, unsigned rank, double v)
{
    asm volatile("st.shared::cluster.f64 [%0], %1;\n" ::"r"(peer_addr(p, rank)), "d"(v) : "memory");
}

// The cluster as one team: cells [lo, hi) belong to this CTA.
struct Team {
    Blk B;
    unsigned rank, size;
    int slice, lo, hi;
    double *xch; // [2][2][16] exchange slots (double-buffered, two values)
    int xb = 0;
    __device__ void sync() const { cl_sync(); }
    // Cluster sums: each CTA's total goes into every CTA's exchange slots,
    // and after the cluster barrier every warp adds the (at most 16) totals
    // with one shuffle tree: the same values in the same order in every warp
    // of every CTA, so all hold bit-identical sums and every loop test
    // agrees. (A sequential add of the totals in every lane cost each warp
    // 16 FP64 instructions per sum.)
    __device__ double sum(double a)
    {
        a = B.sum(a);
        double *s = xch + xb * 32;
        if (threadIdx.x < size) st_peer(s + rank, threadIdx.x, a);
        cl_sync();
        const unsigned lane = threadIdx.x & 31;
        double t = lane < size ? s[lane] : 0.0;
        t = warp_sum(t);
        xb ^= 1;
        return t;
    }
    __device__ void sum2(double &a, double &b)
    {
        B.sum2(a, b);
        double *s = xch + xb * 32;
        if (threadIdx.x < size) {
            st_peer(s + rank, threadIdx.x, a);
            st_peer(s + 16 + rank, threadIdx.x, b);
        }
        cl_sync();
        const unsigned lane = threadIdx.x & 31;
        double ta = lane < size ? s[lane] : 0.0, tb = lane < size ? s[16 + lane] : 0.0;
        warp_sum2(ta, tb);
        a = ta;
        b = tb;
        xb ^= 1;
    }
    // value of slice vector v at cell j (this CTA's or a peer's slice)
    __device__ __forceinline__ double at(const double *v, int j) const
    {
        if (j >= lo && j < hi) return v[j - lo];
        const unsigned o = (unsigned)(j / slice);
        return ld_peer(v + (j - (int)o * slice), o);
    }
};

// Row i (a cell of this CTA) of A D^-1 applied to the slice vector x; m holds
// this CTA's rows of the column-scaled operator, [6][slice].
__device__ __forceinline__ double spmv_row_team(const Team &T, const double *m, const double *x, int i, int n, int nx)
{
    const int li = i - T.lo, s = T.slice;
    double v = x[li];
    const int ix = i % nx;
    if (ix > 0) v += m[s + li] * T.at(x, i - 1);
    if (ix < nx - 1) v += m[2 * s + li] * T.at(x, i + 1);
    if (i >= nx) v += m[3 * s + li] * T.at(x, i - nx);
    if (i + nx < n) v += m[4 * s + li] * T.at(x, i + nx);
    return v;
}

// bicgstab_reg() on the team's slices: each thread's R rows (cells
// lo + threadIdx.x + j blockDim.x) of every vector in registers, p and s
// published in this CTA's shared memory (w, w + slice) for the neighbours,
// in a peer's slice read through distributed shared memory.
template <int R>
__device__ int bicgstab_team_reg(const CmfdView &c, Team &T, const double *m, const double *b, double *x, double tol,
                                 int max_it, double *w, double &rr0)
{
    const int n = c.n_cell, nx = c.nx, s = T.slice, lo = T.lo, hi = T.hi, bd = blockDim.x;
    double *P = w, *S = w + s;
    double xr[R], rr_[R], r0[R], p[R], v[R], bv[R], cw[R], ce[R], cs[R], cn[R];
    bool ok[R];
#pragma unroll
    for (int j = 0; j < R; j++) {
        const int i = lo + (int)threadIdx.x + j * bd, li = i - lo;
        ok[j] = i < hi;
        const int ix = i % nx;
        cw[j] = (ok[j] && ix > 0) ? m[s + li] : 0.0;
        ce[j] = (ok[j] && ix < nx - 1) ? m[2 * s + li] : 0.0;
        cs[j] = (ok[j] && i >= nx) ? m[3 * s + li] : 0.0;
        cn[j] = (ok[j] && i + nx < n) ? m[4 * s + li] : 0.0;
        bv[j] = ok[j] ? b[li] : 0.0;
        xr[j] = ok[j] ? x[li] * m[li] : 0.0;
        p[j] = 0.0;
        v[j] = 0.0;
    }
    // row j applied to the slice vector V (own entry e); absent neighbours
    // are skipped (their entries would be a peer load)
    auto apply = [&](const double *V, int j, double e) {
        const int i = lo + (int)threadIdx.x + j * bd;
        double a = e;
        if (cw[j] != 0.0) a = fma(cw[j], T.at(V, i - 1), a);
        if (ce[j] != 0.0) a = fma(ce[j], T.at(V, i + 1), a);
        if (cs[j] != 0.0) a = fma(cs[j], T.at(V, i - nx), a);
        if (cn[j] != 0.0) a = fma(cn[j], T.at(V, i + nx), a);
        return a;
    };
    auto residual = [&](double &acc) {
#pragma unroll
        for (int j = 0; j < R; j++)
            if (ok[j]) x[threadIdx.x + j * bd] = xr[j];
        T.sync();
#pragma unroll
        for (int j = 0; j < R; j++) {
            const double ri = ok[j] ? bv[j] - apply(x, j, xr[j]) : 0.0;
            rr_[j] = ri;
            r0[j] = ri;
            acc += ri * ri;
        }
    };
    const double eps2 = 2.220446049250313e-16 * 2.220446049250313e-16;
    double rr = 0.0, bb = 0.0;
    residual(rr);
#pragma unroll
    for (int j = 0; j < R; j++) bb += bv[j] * bv[j];
    T.sum2(rr, bb);
    rr0 = rr;
    if (bb == 0.0) {
#pragma unroll
        for (int j = 0; j < R; j++)
            if (ok[j]) x[threadIdx.x + j * bd] = 0.0;
        T.sync();
        return 0;
    }
    double r0_sq = rr, rho = 1.0, alpha = 1.0, om = 1.0;
    const double tol2 = tol * tol * bb;
    int it = 0, restarts = 0;
    double rho_new = rr;
    while (rr > tol2 && it < max_it) {
        double rho_old = rho;
        rho = rho_new;
        if (fabs(rho) < eps2 * r0_sq) {
            T.sync();
            double acc = 0.0;
            residual(acc);
            acc = T.sum(acc);
            rho = r0_sq = acc;
            if (restarts++ == 0) it = 0;
        }
        // Eigen's (rho / rho_old) (alpha / omega) with one division
        const double beta = (rho * alpha) / (rho_old * om);
#pragma unroll
        for (int j = 0; j < R; j++) {
            p[j] = rr_[j] + beta * (p[j] - om * v[j]);
            if (ok[j]) P[threadIdx.x + j * bd] = p[j];
        }
        T.sync();
        double r0v = 0.0;
#pragma unroll
        for (int j = 0; j < R; j++) {
            v[j] = ok[j] ? apply(P, j, p[j]) : 0.0;
            r0v += r0[j] * v[j];
        }
        r0v = T.sum(r0v);
        alpha = rho / r0v;
        double sv[R];
#pragma unroll
        for (int j = 0; j < R; j++) {
            sv[j] = rr_[j] - alpha * v[j];
            if (ok[j]) S[threadIdx.x + j * bd] = sv[j];
        }
        T.sync();
        double tt = 0.0, ts = 0.0, tv[R];
#pragma unroll
        for (int j = 0; j < R; j++) {
            tv[j] = ok[j] ? apply(S, j, sv[j]) : 0.0;
            tt += tv[j] * tv[j];
            ts += tv[j] * sv[j];
        }
        T.sum2(tt, ts);
        om = (tt > 0.0) ? ts / tt : 0.0;
        double nrr = 0.0, nrho = 0.0;
#pragma unroll
        for (int j = 0; j < R; j++) {
            xr[j] += alpha * p[j] + om * sv[j];
            const double ri = sv[j] - om * tv[j];
            rr_[j] = ri;
            nrr += ri * ri;
            nrho += r0[j] * ri;
        }
        T.sum2(nrr, nrho);
        rr = nrr;
        rho_new = nrho;
        it++;
    }
    T.sync();
#pragma unroll
    for (int j = 0; j < R; j++)
        if (ok[j]) x[threadIdx.x + j * bd] = xr[j] * m[5 * s + threadIdx.x + j * bd];
    T.sync();
    return it;
}

// bicgstab() on the team's slices: the same iterates and stopping test.
__device__ int bicgstab_team(const CmfdView &c, Team &T, const double *m, const double *b, double *x, double tol,
                             int max_it, double *w, double &rr0)
{
    switch ((T.hi - T.lo + (int)blockDim.x - 1) / (int)blockDim.x) {
    case 1: return bicgstab_team_reg<1>(c, T, m, b, x, tol, max_it, w, rr0);
    case 2: return bicgstab_team_reg<2>(c, T, m, b, x, tol, max_it, w, rr0);
    default: break;
    }
    const int n = c.n_cell, nx = c.nx, s = T.slice, lo = T.lo, hi = T.hi;
    double *r = w, *r0 = w + s, *p = w + 2 * s, *v = w + 3 * s, *sv = w + 4 * s, *t = w + 5 * s;
    const double eps2 = 2.220446049250313e-16 * 2.220446049250313e-16;
    for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) x[i - lo] *= m[i - lo];
    T.sync();
    double rr = 0.0, bb = 0.0;
    for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
        const int li = i - lo;
        double ri = b[li] - spmv_row_team(T, m, x, i, n, nx);
        r[li] = ri;
        r0[li] = ri;
        p[li] = 0.0;
        v[li] = 0.0;
        rr += ri * ri;
        bb += b[li] * b[li];
    }
    T.sum2(rr, bb);
    rr0 = rr;
    if (bb == 0.0) {
        for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) x[i - lo] = 0.0;
        T.sync();
        return 0;
    }
    double r0_sq = rr, rho = 1.0, alpha = 1.0, om = 1.0;
    const double tol2 = tol * tol * bb;
    int it = 0, restarts = 0;
    double rho_new = rr;
    while (rr > tol2 && it < max_it) {
        double rho_old = rho;
        rho = rho_new;
        if (fabs(rho) < eps2 * r0_sq) {
            T.sync();
            double acc = 0.0;
            for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
                const int li = i - lo;
                double ri = b[li] - spmv_row_team(T, m, x, i, n, nx);
                r[li] = ri;
                r0[li] = ri;
                acc += ri * ri;
            }
            acc = T.sum(acc);
            rho = r0_sq = acc;
            if (restarts++ == 0) it = 0;
        }
        // Eigen's (rho / rho_old) (alpha / omega) with one division
        const double beta = (rho * alpha) / (rho_old * om);
        for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
            const int li = i - lo;
            p[li] = r[li] + beta * (p[li] - om * v[li]);
        }
        T.sync();
        double r0v = 0.0;
        for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
            const int li = i - lo;
            const double vi = spmv_row_team(T, m, p, i, n, nx);
            v[li] = vi;
            r0v += r0[li] * vi;
        }
        r0v = T.sum(r0v);
        alpha = rho / r0v;
        for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
            const int li = i - lo;
            sv[li] = r[li] - alpha * v[li];
        }
        T.sync();
        double tt = 0.0, ts = 0.0;
        for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
            const int li = i - lo;
            const double ti = spmv_row_team(T, m, sv, i, n, nx);
            t[li] = ti;
            tt += ti * ti;
            ts += ti * sv[li];
        }
        T.sum2(tt, ts);
        om = (tt > 0.0) ? ts / tt : 0.0;
        double nrr = 0.0, nrho = 0.0;
        for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
            const int li = i - lo;
            x[li] += alpha * p[li] + om * sv[li];
            double ri = sv[li] - om * t[li];
            r[li] = ri;
            nrr += ri * ri;
            nrho += r0[li] * ri;
        }
        T.sum2(nrr, nrho);
        rr = nrr;
        rho_new = nrho;
        it++;
    }
    T.sync();
    for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) x[i - lo] *= m[5 * s + i - lo];
    T.sync();
    return it;
}

} // namespace

__device__ void cmfd_body_cluster(CmfdView c, int all_groups)
{
    extern __shared__ __align__(16) double sm[];
    const int n = c.n_cell, G = c.G, ns = c.n_surf;
    Team T;
    T.B.nw = blockDim.x >> 5;
    T.B.scratch = sm; // gather_scratch(nw) doubles: the CTA's gathered sums
    T.B.gather = true;
    const int sc = gather_scratch(T.B.nw);
    T.xch = sm + sc; // 64 doubles
    T.rank = cl_rank();
    T.size = cl_nrank();
    T.slice = (n + (int)T.size - 1) / (int)T.size;
    T.lo = min(n, (int)T.rank * T.slice);
    T.hi = min(n, T.lo + T.slice);
    const int s = T.slice, lo = T.lo, hi = T.hi, bd = blockDim.x, tid = threadIdx.x;
    // slice vectors: b, x, 6 BiCGSTAB vectors; the current group's operator rows
    // ms: the current group's rows, or with all_groups every group's rows [G][6][slice]
    double *b = sm + sc + 64, *x = b + s, *w = x + s, *ms = w + 6 * s;
    double k = *c.k;
    if (c.fixup)
        for (int g = 0; g < G; g++)
            for (int i = lo + tid; i < hi; i += bd) c.flux[(size_t)g * n + i] = fmax(c.flux[(size_t)g * n + i], 0.0);
    T.sync();

    // surface coupling coefficients (cmfd.cpp:404-499), surfaces dealt over the cluster
    for (int idx = (int)T.rank * bd + tid; idx < G * ns; idx += (int)T.size * bd) {
        int g = idx / ns, is = idx % ns;
        int c1, c2, nrm;
        surf_info(c, is, c1, c2, nrm);
        int lo_bc = (nrm == X_NORM) ? c.bc[WEST] : (nrm == Y_NORM) ? c.bc[SOUTH] : c.bc[BOTTOM];
        int hi_bc = (nrm == X_NORM) ? c.bc[EAST] : (nrm == Y_NORM) ? c.bc[NORTH] : c.bc[TOP];
        double d1 = (c1 > -1) ? (1.0 / (3.0 * c.xstr[(size_t)c1 * G + g])) / thickness(c, c1, nrm)
                              : (lo_bc == (int)BoundaryType::VACUUM ? 0.5 / 2.0 : 0.0);
        double d2 = (c2 > -1) ? (1.0 / (3.0 * c.xstr[(size_t)c2 * G + g])) / thickness(c, c2, nrm)
                              : (hi_bc == (int)BoundaryType::VACUUM ? 0.5 / 2.0 : 0.0);
        double dt = 2.0 * d1 * d2 / (d1 + d2);
        double stil = (d1 > 0.0) ? d1 / (d1 + d2) : d2 / (d1 + d2);
        double dh = 0.0, sh = 0.0;
        if (nrm != Z_NORM && c.has_radial) {
            double j = c.cur[(size_t)g * ns + is];
            double sfc = c.sflux[(size_t)g * ns + is];
            double fl = c1 >= 0 ? __ldcg(c.flux + (size_t)g * n + c1) : 0.0;
            double fr = c2 >= 0 ? __ldcg(c.flux + (size_t)g * n + c2) : 0.0;
            dh = (j + dt * (fr - fl)) / (fl + fr);
            if (!isfinite(dh)) dh = 0.0;
            sh = (c1 >= 0) ? (sfc - stil * fl - (1.0 - stil) * fr) / (fl + fr) : (sfc - stil * fr) / fr;
        }
        c.d_tilde[idx] = dt;
        c.s_tilde[idx] = stil;
        c.d_hat[idx] = dh;
        c.s_hat[idx] = sh;
    }
    T.sync();
    // 5-point operator per group (cmfd.cpp:506-544), this CTA's rows
    for (int g = 0; g < G; g++)
        for (int i = lo + tid; i < hi; i += bd) {
            const double *dt = c.d_tilde + (size_t)g * ns;
            const double *dh = c.d_hat + (size_t)g * ns;
            double diag = cell_vol(c, i) * c.xsrm[(size_t)i * G + g];
            const int surfs[6] = {EAST, NORTH, WEST, SOUTH, TOP, BOTTOM};
            for (int k6 = 0; k6 < 6; k6++) {
                int sd = surfs[k6];
                int sf = coarse_surf(c, i, sd);
                double h = __ldcg(dh + sf);
                if (sd == WEST || sd == SOUTH || sd == BOTTOM) h = -h;
                diag += area(c, i, sd) * (__ldcg(dt + sf) + h);
            }
            double *m = c.mat + (size_t)g * 6 * n;
            m[i] = (diag != 0.0) ? diag : 1.0;
            m[(size_t)5 * n + i] = (diag != 0.0) ? 1.0 / diag : 1.0; // Jacobi preconditioner
            const int offs[4] = {WEST, EAST, SOUTH, NORTH};
            for (int q = 0; q < 4; q++) {
                int sd = offs[q];
                double v = 0.0;
                if (neighbor(c, i, sd) >= 0) {
                    int sf = coarse_surf(c, i, sd);
                    double h = __ldcg(dh + sf);
                    if (sd == WEST || sd == SOUTH) h = -h;
                    v = area(c, i, sd) * (h - __ldcg(dt + sf));
                }
                m[(size_t)(q + 1) * n + i] = v;
            }
        }
    T.sync();
    // column scaling by the neighbour's inverse diagonal (neighbours' rows may be a peer's)
    for (int g = 0; g < G; g++)
        for (int i = lo + tid; i < hi; i += bd) {
            const int ix = i % c.nx;
            double *m = c.mat + (size_t)g * 6 * n;
            const double *dinv = m + (size_t)5 * n;
            if (ix > 0) m[(size_t)n + i] *= __ldcg(dinv + i - 1);
            if (ix < c.nx - 1) m[(size_t)2 * n + i] *= __ldcg(dinv + i + 1);
            if (i >= c.nx) m[(size_t)3 * n + i] *= __ldcg(dinv + i - c.nx);
            if (i + c.nx < n) m[(size_t)4 * n + i] *= __ldcg(dinv + i + c.nx);
        }
    T.sync();
    if (all_groups)
        for (int g = 0; g < G; g++)
            for (int q = 0; q < 6; q++)
                for (int i = lo + tid; i < hi; i += bd)
                    ms[((size_t)g * 6 + q) * s + i - lo] = c.mat[((size_t)g * 6 + q) * n + i];

    // fission source (own cells) and total fission (own cells' share)
    auto fis_src = [&](double kk) {
        for (int i = lo + tid; i < hi; i += bd)
            c.fs[i] = group_dot(c.xsnf + (size_t)i * G, 1, c.flux + i, n, G, -1) * (1.0 / kk);
    };
    auto tot_fis = [&]() {
        double f = 0.0;
        for (int i = lo + tid; i < hi; i += bd) f += group_dot(c.xsnf + (size_t)i * G, 1, c.flux + i, n, G, -1);
        return f;
    };
    auto source = [&](int g) {
        for (int i = lo + tid; i < hi; i += bd) {
            double sv = c.xsch[(size_t)i * G + g] * c.fs[i];
            sv += group_dot(c.scat + ((size_t)i * G + g) * G, 1, c.flux + i, n, G, g);
            b[i - lo] = sv * cell_vol(c, i);
        }
    };
    fis_src(k);
    double tfis = T.sum(tot_fis());
    double r0 = 0.0;
    for (int g = 0; g < G; g++) {
        source(g);
        // ||M_g x - b_g||^2 with x the group flux (A_ij = m_ij d_j off the diagonal)
        const double *m = c.mat + (size_t)g * 6 * n;
        const double *xg = c.flux + (size_t)g * n;
        double acc = 0.0;
        for (int i = lo + tid; i < hi; i += bd) {
            const int ix = i % c.nx;
            double v = m[i] * xg[i];
            if (ix > 0) v += m[n + i] * (__ldcg(m + i - 1) * __ldcg(xg + i - 1));
            if (ix < c.nx - 1) v += m[2 * n + i] * (__ldcg(m + i + 1) * __ldcg(xg + i + 1));
            if (i >= c.nx) v += m[3 * n + i] * (__ldcg(m + i - c.nx) * __ldcg(xg + i - c.nx));
            if (i + c.nx < n) v += m[4 * n + i] * (__ldcg(m + i + c.nx) * __ldcg(xg + i + c.nx));
            const double d = v - b[i - lo];
            acc += d * d;
        }
        r0 += T.sum(acc);
    }
    r0 = sqrt(r0) / (double)(n * G);
    const double tol = c.resid_reduction * r0;

    int iter = 0, bic_its = 0;
    double psi_err = 1.0, ri = 0.0, k_old = k;
    while (true) {
        iter++;
        for (int i = lo + tid; i < hi; i += bd) c.fs_old[i] = c.fs[i];
        fis_src(k);
        double tfis_old = tfis;
        ri = 0.0;
        for (int g = 0; g < G; g++) {
            const double *mg = c.mat + (size_t)g * 6 * n;
            double *fg = c.flux + (size_t)g * n;
            T.sync();
            const double *mrows = ms + (all_groups ? (size_t)g * 6 * s : 0);
            if (!all_groups)
                for (int q = 0; q < 6; q++)
                    for (int i = lo + tid; i < hi; i += bd) ms[q * s + i - lo] = mg[(size_t)q * n + i];
            source(g);
            for (int i = lo + tid; i < hi; i += bd) x[i - lo] = fg[i];
            T.sync();
            double rr0 = 0.0;
            bic_its += bicgstab_team(c, T, mrows, b, x, tol, 150, w, rr0);
            ri += rr0;
            for (int i = lo + tid; i < hi; i += bd) fg[i] = x[i - lo];
        }
        T.sync();
        ri = sqrt(ri) / (double)(n * G);
        tfis = T.sum(tot_fis());
        k_old = k;
        k = k * tfis / tfis_old;
        double pe = 0.0;
        for (int i = lo + tid; i < hi; i += bd) {
            double e = c.fs[i] - c.fs_old[i];
            pe += e * e;
        }
        psi_err = sqrt(T.sum(pe));
        if ((fabs(k - k_old) < c.k_tol && psi_err < c.psi_tol && ri / r0 < c.resid_reduction) || iter > c.max_iter)
            break;
    }
    for (int g = 0; g < G; g++)
        for (int i = lo + tid; i < hi; i += bd)
            if (c.flux[(size_t)g * n + i] < 0.0) c.flux[(size_t)g * n + i] = -c.flux[(size_t)g * n + i];
    T.sync();
    if (T.rank == 0 && tid == 0) {
        *c.k = k;
        c.stats[0] = iter;
        c.stats[1] = r0;
        c.stats[2] = ri / r0;
        c.stats[3] = psi_err;
        c.stats[4] = bic_its;
        if (!isfinite(k)) atomicOr(c.status, (unsigned)DEV_NAN);
    }
}

__global__ void __launch_bounds__(512, 1) kc_cmfd_solve(CmfdView c, int all_groups)
{
    cmfd_body_cluster(c, all_groups);
}

__global__ void __launch_bounds__(512, 1) k_cmfd_solve(CmfdView c, int vec_in_smem) { cmfd_body(c, vec_in_smem); }

// One CTA per active solve of a batch; the coarse-current flag and the CMFD
// iteration count live in each solve's scalar block.
__global__ void __launch_bounds__(512) kb_cmfd_solve(BatchViews b, int vec_in_smem)
{
    if ((int)blockIdx.x >= *b.n_act) return;
    const int slot = b.act[blockIdx.x];
    CmfdView c = b.cv[slot];
    if (c.red[RED_DONE] != 0.0) return; // finished: frozen
    c.has_radial = (c.red[RED_HAS_RADIAL] != 0.0) ? 1 : 0;
    cmfd_body(c, vec_in_smem); // the CTA's shared memory is sized for the largest mesh of the batch
    if (threadIdx.x == 0) c.red[RED_CMFD_ITS] += c.stats[0];
}

void note_launch_external();

// Warps per CMFD CTA. One warp reaches only about a quarter of an SM's FP64
// rate (one of four schedulers issues), so meshes with work for more than
// one warp get at least four; tiny meshes stay on one warp, where every
// reduction is a shuffle tree. With gathered sums a CTA of about two rows
// per lane does best on the 289-cell assembly (measured per solve: 4 warps
// 180 ms, 5 warps 167 ms, 10 warps 215 ms).
#ifndef MOCGPU_CMFD_CELLS_PER_WARP
#define MOCGPU_CMFD_CELLS_PER_WARP 64
#endif
static int cmfd_warps(int n_cell)
{
    if (n_cell <= 64) return 1;
    int nw = (n_cell + MOCGPU_CMFD_CELLS_PER_WARP - 1) / MOCGPU_CMFD_CELLS_PER_WARP;
    return nw < 4 ? 4 : (nw > 16 ? 16 : nw);
}
// Warps per CTA of the cluster solve: as for one CTA, about two rows per
// lane (MOCGPU_CMFD_CLUSTER_CELLS_PER_WARP), at least four.
#ifndef MOCGPU_CMFD_CLUSTER_CELLS_PER_WARP
#define MOCGPU_CMFD_CLUSTER_CELLS_PER_WARP 64
#endif
static int cluster_warps(int slice)
{
    int nw = (slice + MOCGPU_CMFD_CLUSTER_CELLS_PER_WARP - 1) / MOCGPU_CMFD_CLUSTER_CELLS_PER_WARP;
    return nw < 4 ? 4 : (nw > 16 ? 16 : nw);
}

#ifndef MOCGPU_BATCH_CMFD_ALL_GROUPS
#define MOCGPU_BATCH_CMFD_ALL_GROUPS 1
#endif

// Shared-memory mode of a CMFD CTA: 3 = work vectors and every group's
// operator (only when `all_groups` > 0 groups are asked for: a single solve,
// whose CTA has its SM to itself), 2 = work vectors and the current group's
// operator, 1 = work vectors only, 0 = nothing (vectors in global memory).
static int cmfd_smem_mode(int n_cell, size_t *bytes, int all_groups = 0)
{
    const size_t base = gather_scratch(cmfd_warps(n_cell)) * sizeof(double), lim = 200 * 1024;
    const size_t vec = (size_t)10 * n_cell * sizeof(double), op = (size_t)6 * n_cell * sizeof(double);
    if (all_groups > 0 && base + vec + op * all_groups <= lim) {
        *bytes = base + vec + op * all_groups;
        return 3;
    }
    int mode = (base + vec + op <= lim) ? 2 : (base + vec <= lim) ? 1 : 0;
    *bytes = base + (mode >= 1 ? vec : 0) + (mode == 2 ? op : 0);
    return mode;
}

void launch_b_cmfd(const BatchViews &b, cudaStream_t s)
{
    const int max_cell = b.max_cell;
    const int nw = cmfd_warps(max_cell);
    size_t smem = 0;
    // every group's operator in shared memory too when it fits (measured on
    // the 256-case batch: 209 -> 187 ms of replay time in one engine, 1222 ->
    // 1267 solves/s over four lanes, although the CTAs leave less room for
    // other lanes' sweep CTAs on their SMs)
    const int in_smem = cmfd_smem_mode(max_cell, &smem, MOCGPU_BATCH_CMFD_ALL_GROUPS ? b.max_g : 0);
    ensure_smem_limit((const void *)kb_cmfd_solve, smem);
    note_launch_external();
    kb_cmfd_solve<<<b.cap, 32 * nw, smem, s>>>(b, in_smem);
}

// Meshes above MOCGPU_CMFD_CLUSTER_MIN cells are solved by a cluster of CTAs,
// one slice of about MOCGPU_CMFD_CLUSTER_CELLS cells each (at most 8 CTAs).
// Measured on the 17x17 assembly (289 cells): one CTA 188 ms per solve,
// clusters of 2, 3, 4 and 8 CTAs 228, 195, 198 and 248 ms (the cluster
// barriers and remote reads outweigh the FP64 work they spread); on the
// 68x68 mini-core (4624 cells) a cluster of 8 takes the solve from 4.6 s to
// 1.40 s, 16 CTAs with every group's operator rows in shared memory to
// 1.35 s (1, 2, 8 or 16 warps per CTA instead of 4: 2.9, 2.0, 1.7 and 3.2 s).
#ifndef MOCGPU_CMFD_CLUSTER_MIN
#define MOCGPU_CMFD_CLUSTER_MIN 1024
#endif
#ifndef MOCGPU_CMFD_CLUSTER_CELLS
#define MOCGPU_CMFD_CLUSTER_CELLS 128
#endif
#ifndef MOCGPU_CMFD_CLUSTER_MAX
#define MOCGPU_CMFD_CLUSTER_MAX 16 // CTAs per cluster; above 8 is a non-portable size, checked per launch
#endif
#ifndef MOCGPU_CMFD_CLUSTER_WARPS
#define MOCGPU_CMFD_CLUSTER_WARPS 0 // warps per CTA, 0: from the slice size
#endif
constexpr int kClusterCmfdMinCells = MOCGPU_CMFD_CLUSTER_MIN;

// Cluster shape of a mesh: CTAs, warps per CTA, shared bytes, and whether
// every group's operator rows fit in shared memory.
struct ClusterShape {
    int cl, nw, all_groups;
    size_t smem;
};
static ClusterShape cluster_shape(const CmfdView &c, int max_cl)
{
    ClusterShape sh;
    sh.cl = std::max(2, std::min(max_cl, (c.n_cell + MOCGPU_CMFD_CLUSTER_CELLS - 1) / MOCGPU_CMFD_CLUSTER_CELLS));
    const int slice = (c.n_cell + sh.cl - 1) / sh.cl;
    sh.nw = MOCGPU_CMFD_CLUSTER_WARPS > 0 ? MOCGPU_CMFD_CLUSTER_WARPS : cluster_warps(slice);
    const size_t head = (size_t)gather_scratch(sh.nw) + 64; // gathered sums + the cluster exchange slots
    const size_t lim = 200 * 1024, all = (head + 8 * slice + 6 * c.G * slice) * sizeof(double);
    sh.all_groups = all <= lim ? 1 : 0;
    sh.smem = sh.all_groups ? all : (head + 14 * slice) * sizeof(double);
    return sh;
}

static cudaLaunchConfig_t cluster_config(const ClusterShape &sh, cudaStream_t s, cudaLaunchAttribute *attr)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(sh.cl);
    cfg.blockDim = dim3(32 * sh.nw);
    cfg.dynamicSmemBytes = sh.smem;
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = sh.cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

static void launch_cmfd_cluster(const CmfdView &c, cudaStream_t s)
{
    ensure_smem_limit((const void *)kc_cmfd_solve, 200 * 1024);
    if (MOCGPU_CMFD_CLUSTER_MAX > 8)
        raise_func_attr((const void *)kc_cmfd_solve, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    ClusterShape sh = cluster_shape(c, MOCGPU_CMFD_CLUSTER_MAX);
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_config(sh, s, attr);
    if (sh.cl > 8) {
        // a cluster above the portable 8 CTAs only where this GPU can place one
        int fits = 0;
        if (cudaOccupancyMaxActiveClusters(&fits, kc_cmfd_solve, &cfg) != cudaSuccess || fits < 1) {
            (void)cudaGetLastError();
            sh = cluster_shape(c, 8);
            cfg = cluster_config(sh, s, attr);
        }
    }
    if (sh.smem > 200 * 1024) throw Error(21, "CMFD mesh too large for the cluster solve");
    note_launch_external();
    MOCGPU_CUDA(cudaLaunchKernelEx(&cfg, kc_cmfd_solve, c, sh.all_groups));
}

void launch_cmfd_solve(const CmfdView &c, cudaStream_t s)
{
    if (c.n_cell > kClusterCmfdMinCells) {
        launch_cmfd_cluster(c, s);
        return;
    }
    const int nw = cmfd_warps(c.n_cell);
    size_t smem = 0;
    const int in_smem = cmfd_smem_mode(c.n_cell, &smem, c.G);
    ensure_smem_limit((const void *)k_cmfd_solve, smem);
    note_launch_external();
    k_cmfd_solve<<<1, 32 * nw, smem, s>>>(c, in_smem);
}

} // namespace mocgpu

// ---------------------------------------------------------------------------
// CMFD solve with its work vectors in a fixed module-scope array instead of
// the handle's buffer: no allocation happens on any call. The array holds the
// ten work vectors (right-hand side, group flux copy, eight BiCGSTAB vectors)
// of meshes up to kStaticCmfdMaxCells coarse cells. The kernel writes every
// entry it reads (BiCGSTAB zeroes its p and v itself), so nothing in the
// array has to start at zero. All calls in the process share the array:
// calls that overlap in time on the same device race on it.
namespace mocgpu {

constexpr int kStaticCmfdMaxCells = 8192;
static __device__ __align__(256) double g_cmfd_static_scratch[10 * kStaticCmfdMaxCells];

__global__ void __launch_bounds__(512) k_cmfd_solve_static(CmfdView c) { cmfd_body(c, 0); }

// Device address of the array, looked up once per device (with that device
// current) on the first call that runs there.
static double *static_scratch_address()
{
    static std::mutex mu;
    static double *addr[64] = {nullptr};
    int dev = 0;
    MOCGPU_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw Error(20, "device ordinal out of range for the static CMFD scratch");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_cmfd_static_scratch);
        if (e != cudaSuccess)
            throw Error(20, std::string("cudaGetSymbolAddress of the static CMFD scratch failed: ") +
                                cudaGetErrorString(e));
        addr[dev] = static_cast<double *>(p);
    }
    return addr[dev];
}

int static_cmfd_max_cells() { return kStaticCmfdMaxCells; }

void launch_cmfd_solve_static(const CmfdView &c, cudaStream_t s)
{
    if (c.n_cell > kStaticCmfdMaxCells)
        throw Error(21, "coarse mesh has " + std::to_string(c.n_cell) + " cells; the static CMFD scratch holds " +
                            std::to_string(kStaticCmfdMaxCells));
    CmfdView v = c;
    v.vec = static_scratch_address();
    const int nw = cmfd_warps(c.n_cell);
    note_launch_external();
    k_cmfd_solve_static<<<1, 32 * nw, gather_scratch(nw) * sizeof(double), s>>>(v);
}

} // namespace mocgpu

// ---------------------------------------------------------------------------
// Incoming boundary angular flux from the CMFD solution
// (MoCSweeper::update_incoming_flux, moc_sweeper.cpp:255-291, reading the
// partial currents of CMFD::store_currents, cmfd.cpp:555-638). Off unless the
// solve's options ask for it, as in MOCC, whose call of it is commented out
// (eigen_solver.cpp:289).
namespace mocgpu {

namespace {

// CMFD::store_currents: net current and surface flux of every surface from
// the solved coarse flux, and the two partial currents from them. Of the
// partial currents the update reads only 2 (J+ + J-); that is stored per
// [G][n_surf], the previous solve's values moving to part_old first.
__device__ __forceinline__ void store_partial(const CmfdView &c, double *part, double *part_old, int idx)
{
    const int ns = c.n_surf, n = c.n_cell;
    const int g = idx / ns, is = idx % ns;
    int c1, c2, nrm;
    surf_info(c, is, c1, c2, nrm);
    const double fr = c2 >= 0 ? c.flux[(size_t)g * n + c2] : 0.0;
    const double fl = c1 >= 0 ? c.flux[(size_t)g * n + c1] : 0.0;
    const double dt = c.d_tilde[idx], dh = c.d_hat[idx], st = c.s_tilde[idx], sh = c.s_hat[idx];
    const double j = -dt * (fr - fl) + dh * (fr + fl);
    const double sf = (c1 >= 0) ? st * fl + (1.0 - st) * fr + sh * (fl + fr) : st * fr + sh * (fl + fr);
    const double jp = 0.25 * sf + 0.5 * j, jm = 0.25 * sf - 0.5 * j;
    part_old[idx] = part[idx];
    part[idx] = 2.0 * (jp + jm);
}
__global__ void k_store_partials(CmfdView c, double *part, double *part_old)
{
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < c.G * c.n_surf; idx += gridDim.x * blockDim.x)
        store_partial(c, part, part_old, idx);
}

// One boundary entry: scaled by the change of 2 (J+ + J-) on its surface
// since the previous CMFD solve, or (first solve) set to the isotropic
// angular flux 2 (J+ + J-) / 4pi.
__device__ __forceinline__ double incoming_value(double in, const double *part, const double *part_old, int idx,
                                                 int has_old)
{
    if (has_old) {
        const double old = part_old[idx];
        return old > 0.0 ? in * (part[idx] / old) : in;
    }
    return (2.0 / (4.0 * 3.1415926535897932)) * (0.5 * part[idx]);
}

// Which surface a boundary entry reads, and whether it is left alone:
// mode 1 reads the partial currents at the index of the track's starting
// coarse cell as MOCC's update_incoming_generic does (moc_sweeper.hpp:
// 198-233: ray.cm_cell_fw() passed where a surface index is taken, which
// lands on the cell's bottom z-face); mode 2 reads the core-boundary surface
// the track enters through and leaves entries on vacuum faces at zero.
__device__ __forceinline__ int entry_surface(const CmfdView &c, int cell, int surf, int mode)
{
    if (mode == 1) return (cell >= 0 && cell < c.n_surf) ? cell : -1;
    if (surf < 0 || surf >= c.n_surf) return -1;
    int c1, c2, nrm;
    surf_info(c, surf, c1, c2, nrm);
    int face = (nrm == X_NORM) ? (c1 < 0 ? WEST : EAST) : (nrm == Y_NORM) ? (c1 < 0 ? SOUTH : NORTH) : -1;
    if (face < 0 || (c1 >= 0 && c2 >= 0)) return -1;
    return c.bc[face] == (int)BoundaryType::VACUUM ? -1 : surf;
}

// update_incoming_generic: every (group, track, polar angle) rewrites the two
// boundary entries its track starts from, forward and backward. Each entry
// is the start of exactly one track in its direction, so no two threads
// write the same entry.
template <typename Real>
__device__ void incoming_update(const GeomView &gv, const CmfdView &c, Real *psi_in, const double *part,
                                const double *part_old, int mode, int has_old)
{
    const int per_g = gv.n_tracks * gv.pol;
    const int total = gv.G * per_g;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int g = idx / per_g, r = idx % per_g, t = r / gv.pol, p = r % gv.pol;
        const SetPolar &sp = gv.sp[gv.trk_set[t] * gv.pol + p];
        const int4 e = gv.trk_entry[t];
        Real *psi = psi_in + (size_t)g * gv.bc_per_group;
        const int s1 = entry_surface(c, e.x, e.z, mode), s2 = entry_surface(c, e.y, e.w, mode);
        const size_t gs = (size_t)g * c.n_surf;
        if (s1 >= 0) {
            Real &v = psi[gv.bc_off[sp.ang_fwd] + gv.trk_bc0[t]];
            v = (Real)incoming_value((double)v, part + gs, part_old + gs, s1, has_old);
        }
        if (s2 >= 0) {
            Real &v = psi[gv.bc_off[sp.ang_bwd] + gv.trk_bc1[t]];
            v = (Real)incoming_value((double)v, part + gs, part_old + gs, s2, has_old);
        }
    }
}
template <typename Real>
__global__ void k_incoming_update(GeomView gv, CmfdView c, Real *psi_in, const double *part, const double *part_old,
                                  int mode, int has_old)
{
    incoming_update<Real>(gv, c, psi_in, part, part_old, mode, has_old);
}

// Batched forms, one solve per blockIdx.y (solves that ended are frozen):
// the partial currents of each solve's CMFD solution, the boundary-flux
// update (a previous CMFD solve's currents exist once RED_CMFD_SOLVES > 0),
// then the count of CMFD solves.
__global__ void kb_store_partials(BatchViews b)
{
    if ((int)blockIdx.y >= *b.n_act) return;
    const int slot = b.act[blockIdx.y];
    const StateView &st = b.sv[slot];
    if (st.red[RED_DONE] != 0.0) return;
    const CmfdView &c = b.cv[slot];
    const int n1 = c.G * c.n_surf;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n1; idx += gridDim.x * blockDim.x)
        store_partial(c, st.part, st.part + n1, idx);
}
template <typename Real> __global__ void kb_incoming_update(BatchViews b, int mode)
{
    if ((int)blockIdx.y >= *b.n_act) return;
    const int slot = b.act[blockIdx.y];
    const StateView &st = b.sv[slot];
    if (st.red[RED_DONE] != 0.0) return;
    const CmfdView &c = b.cv[slot];
    const double *part = st.part;
    incoming_update<Real>(b.gv[slot], c, (Real *)st.psi_in, part, part + (size_t)c.G * c.n_surf, mode,
                          st.red[RED_CMFD_SOLVES] > 0.0 ? 1 : 0);
}
__global__ void kb_count_cmfd(BatchViews b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *b.n_act) return;
    double *red = b.sv[b.act[i]].red;
    if (red[RED_DONE] == 0.0) red[RED_CMFD_SOLVES] += 1.0;
}

} // namespace

void launch_b_incoming_update(const BatchViews &b, int precision, int mode, cudaStream_t s)
{
    if (mode != 1 && mode != 2) throw Error(1, "incoming update mode must be 1 (MOCC) or 2 (entry surface)");
    note_launch_external();
    kb_store_partials<<<dim3((unsigned)((b.max_surf * b.max_g + 255) / 256), (unsigned)b.cap), 256, 0, s>>>(b);
    note_launch_external();
    if (precision == 0) kb_incoming_update<double><<<dim3(64, (unsigned)b.cap), 256, 0, s>>>(b, mode);
    else kb_incoming_update<float><<<dim3(64, (unsigned)b.cap), 256, 0, s>>>(b, mode);
    note_launch_external();
    kb_count_cmfd<<<(b.cap + 127) / 128, 128, 0, s>>>(b);
}

void launch_incoming_update(const GeomView &gv, const CmfdView &c, void *psi_in, int precision, double *part,
                            int mode, int has_old, cudaStream_t s)
{
    if (mode != 1 && mode != 2) throw Error(1, "incoming update mode must be 1 (MOCC) or 2 (entry surface)");
    const int n1 = c.G * c.n_surf;
    note_launch_external();
    k_store_partials<<<(n1 + 255) / 256, 256, 0, s>>>(c, part, part + (size_t)n1);
    launch_apply_incoming(gv, c, psi_in, precision, part, mode, has_old, s);
}

void launch_apply_incoming(const GeomView &gv, const CmfdView &c, void *psi_in, int precision, const double *part,
                           int mode, int has_old, cudaStream_t s)
{
    if (mode != 1 && mode != 2) throw Error(1, "incoming update mode must be 1 (MOCC) or 2 (entry surface)");
    const double *part_old = part + (size_t)c.G * c.n_surf;
    const int64_t n2 = (int64_t)gv.G * gv.n_tracks * gv.pol;
    const int blocks = (int)std::min<int64_t>((n2 + 255) / 256, 152 * 16);
    note_launch_external();
    if (precision == 0)
        k_incoming_update<double><<<blocks, 256, 0, s>>>(gv, c, static_cast<double *>(psi_in), part, part_old, mode,
                                                         has_old);
    else
        k_incoming_update<float><<<blocks, 256, 0, s>>>(gv, c, static_cast<float *>(psi_in), part, part_old, mode,
                                                        has_old);
}

} // namespace mocgpu
