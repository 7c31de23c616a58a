// Bundled work-unit MoC sweep: device code and kernel templates, shared by
// the translation units that instantiate it (sweep_fast.cu: the single-solve
// kernel and the default shape of the batched kernel; sweep_fast_shapes_*.cu:
// the FP32 batched kernel in the other streaming shapes).
//
// Bundled work-unit MoC sweep (the sweep of moc_sweeper_kernel.inc.hpp:36-180,
// rearranged for the GPU).
//
// One CTA per work unit (a few bundles of 32 tracks of one azimuthal set).
// The unit's FSR cross sections and sources are staged into shared memory as
// (Sigma_t, qbar) pairs and the unit's FSR tally lives in shared memory
// (fixed point in the FP32 path, see tally_fixed). One warp sweeps one bundle
// in one direction, one track per lane, all polar angles of the azimuth in
// registers (the forward and the backward pass of a bundle run on two warps,
// each a template instance of its own). Each warp streams its bundle's
// segment rows through a shared-memory ring with 16-byte cp.async copies,
// the next chunk landing while the current one is swept. After the bundles,
// the unit's tally is added to the global FSR tally with one atomic per
// touched FSR. The single-solve kernel launches one CTA per unit of a phase;
// the batched kernel is persistent over the (solve, unit) items of all
// active solves.
#pragma once

#include <algorithm>
#include <climits>

#include "kernels.cuh"

namespace mocgpu {

__device__ __forceinline__ double att_fast(double tau, const double *tab)
{
    // MOCC's table exponential (exponential.hpp:56-112): [-10, 0], 10000 intervals
    double v = -tau;
    if (v < -10.0 || v > 0.0) return 1.0 - exp(v);
    const double rspace = 1000.0, space = 1.0e-3;
    int i = (int)((v + 10.0) * rspace);
    if (i >= kExpN) i = kExpN - 1;
    v -= space * i - 10.0;
    double d0 = __ldg(tab + i), d1 = __ldg(tab + i + 1);
    return 1.0 - (d0 + (d1 - d0) * v * rspace);
}
// 1 - e^{-tau} in FP32 from the identity e^{-tau} = 2^{-tau log2 e}, with
// the hardware base-2 exponential (ex2.approx, relative error about 2^-22).
// The absolute error of the difference is about one ulp of 1.0 (6e-8) for
// every tau, the size of the FP32 rounding of the angular-flux update it
// feeds and below the interpolation error of MOCC's FP64 table (h^2/8 =
// 1.25e-7). `ntau_l2` is -tau * log2(e).
__device__ __forceinline__ float att_exp2(float ntau_l2)
{
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(ntau_l2));
    return 1.0f - e;
}


// Attenuation 1 - e^{-tau0 / sin(theta)} of one polar angle; `rs` is the
// per-polar factor prepared by polar_factor().
__device__ __forceinline__ double atten(double tau0, double rs, const double *tab) { return att_fast(tau0 * rs, tab); }
__device__ __forceinline__ float atten(float tau0, float rs, const double *) { return att_exp2(tau0 * rs); }
template <typename Real> __device__ __forceinline__ Real polar_factor(double rsin)
{
    return sizeof(Real) == 4 ? (Real)(-rsin * 1.4426950408889634) : (Real)rsin; // FP32: -log2(e)/sin
}

template <typename Real> struct Pair;
template <> struct Pair<float> {
    using T = float2;
};
template <> struct Pair<double> {
    using T = double2;
};
// Chunk shape of the segment rings (build-time: -DMOCGPU_SWEEP_ROWS=...,
// -DMOCGPU_SWEEP_STAGES=...) and rows per unrolled step.
#ifndef MOCGPU_SWEEP_ROWS
#define MOCGPU_SWEEP_ROWS 8
#endif
#ifndef MOCGPU_SWEEP_STAGES
#define MOCGPU_SWEEP_STAGES 2
#endif
#ifndef MOCGPU_TALLY_BITS
#define MOCGPU_TALLY_BITS 50
#endif
#ifndef MOCGPU_SWEEP_UNROLL
#define MOCGPU_SWEEP_UNROLL 4
#endif
// -DMOCGPU_SWEEP_MINB=n: the batched kernel (at most 256 threads) is built
// for n resident CTAs of 256 threads per SM (a register cap)
#if defined(MOCGPU_SWEEP_MINB) && MOCGPU_SWEEP_MINB > 0
#define MOCGPU_SWEEP_BOUNDS __launch_bounds__(256, MOCGPU_SWEEP_MINB)
#else
#define MOCGPU_SWEEP_BOUNDS
#endif
// The fixed-point tally's words cannot wrap: a contribution below
// 2^TALLY_BITS / max_hits adds less than 2^(TALLY_BITS - 20) / max_hits + 1 to
// the signed high word and less than 2^20 to the unsigned low word, so
// max_hits adds keep the high word below 2^(TALLY_BITS - 20) + max_hits and
// the low word below max_hits * 2^20. Both must stay inside 32-bit words.
static_assert(MOCGPU_TALLY_BITS - 20 <= 30, "fixed-point tally: the high word would overflow");
static_assert((long long)kMaxTallyHits * (1ll << 20) <= (1ll << 31), "fixed-point tally: the low word would wrap");
static_assert((1ll << (MOCGPU_TALLY_BITS - 20)) + kMaxTallyHits < (1ll << 31),
              "fixed-point tally: the high word would overflow");
template <typename Real> struct Chunk {
    static constexpr int tally_copies = 2; // FP64 shared tallies, lane l adds into copy l % tally_copies
    static constexpr bool fixed = sizeof(Real) == 4; // FP32: two-word fixed-point tally (same bytes)
};
// Streaming shape of a warp's segment ring: rows per chunk, chunks in flight,
// rows per unrolled step. The single-solve kernel and the FP64 batched kernel
// use the default; the FP32 batched kernel is also built in the shapes of
// kSweepShapes (the autotuner picks one per engine).
template <int ROWS, int STAGES, int UNROLL> struct Shape {
    static constexpr int rows = ROWS, stages = STAGES, unroll = UNROLL;
    static_assert(ROWS % UNROLL == 0 && STAGES >= 2, "sweep shape");
};
using DefaultShape = Shape<MOCGPU_SWEEP_ROWS, MOCGPU_SWEEP_STAGES, MOCGPU_SWEEP_UNROLL>;
// The batched sweep's shapes: 0 the default, then shorter and longer chunks
// and deeper rings. ShapeN<i> is a type of its own per index, so every kernel
// instance belongs to exactly one translation unit.
constexpr int kShapeRows[kSweepShapeCount] = {MOCGPU_SWEEP_ROWS, 4, 4, 16, 8};
constexpr int kShapeStages[kSweepShapeCount] = {MOCGPU_SWEEP_STAGES, 2, 4, 2, 3};
template <int I> struct ShapeN : Shape<kShapeRows[I], kShapeStages[I], MOCGPU_SWEEP_UNROLL> {};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Shared bytes per unit FSR: the (Sigma_t, qbar) pair and the tally (FP32:
// fixed-point high and low words; FP64: the tally copies).
template <typename Real> __host__ __device__ constexpr size_t fsr_slot_bytes()
{
    return sizeof(Real) == 4 ? 2 * sizeof(float) + 2 * 4 : (2 + Chunk<Real>::tally_copies) * sizeof(Real);
}

// Bytes of one warp's ring buffer (the chunks in flight of lengths and local FSR ids).
template <typename Real, class SH> __host__ __device__ constexpr size_t ring_bytes()
{
    return (size_t)SH::stages * SH::rows * (32 * sizeof(Real) + 32 * sizeof(uint16_t));
}

// FP64 path: adds each lane's contribution to the shared tally. A float add
// on shared memory is a compare-and-swap loop, and lanes of a bundle may cross
// the same FSR in the same row; even and odd lanes therefore add into two
// copies of the tally (summed when the unit ends). Padding lanes carry a zero
// contribution and skip the add.
template <typename Real> __device__ __forceinline__ void tally_add(Real *s_tal, int l, Real acc)
{
    if (acc != (Real)0) atomicAdd(s_tal + l, acc);
}

// FP32 path: the unit's tally is fixed point, two 32-bit words per FSR (a
// signed high word counting 2^20 and an unsigned low word), added with
// shared-memory integer atomics. Those are single native operations (a float
// add on shared memory is a compare-and-swap loop that retries and serialises
// the lanes of a warp crossing the same FSR in the same row), they commute,
// and nothing waits on them. A contribution x, already multiplied by the
// unit's power-of-two scale (folded into the polar weights), is an integer
// when |x| >= 2^23 (24 significant bits) and is split exactly as
// x = hi * 2^20 + lo with hi = floor(x / 2^20) and 0 <= lo < 2^20. The scale
// makes |x| < 2^50 / max_hits, so at most max_hits adds keep the high word
// within 2^30 + max_hits and the low word below max_hits * 2^20 <= 2^31.
// Smaller contributions, more than 2^27 / max_hits below the unit's bound
// (fluxes many decades below the unit's largest, as deep in a reflector
// next to a vacuum face), are added straight to the FSR's FP32 tally in
// global memory (a native float reduction), so every contribution keeps its
// FP32 precision. The float compare-and-swap tally
// this replaced was itself faster than merging colliding lanes with
// shuffles first, match-any de-duplication, per-warp copies and global
// float reductions.
__device__ __forceinline__ void tally_fixed(int *s_hi, unsigned *s_lo, float *tally, const int *lf, float inv, int l,
                                            float xs)
{
    if (fabsf(xs) >= 0x1p23f) {
        // 2^23 <= |xs| < 2^50 is an integer: the split is exact, in FP32 and
        // 32-bit conversions (a 64-bit conversion would run on the FP64 pipe)
        const float hf = floorf(xs * 0x1p-20f);
        atomicAdd(s_hi + l, (int)hf);
        atomicAdd(s_lo + l, (unsigned)(int)fmaf(hf, -0x1p20f, xs));
    } else if (xs != 0.f) {
        atomicAdd(tally + lf[l], xs * inv); // below 2^23 units (rare): straight to the FSR's FP32 tally
    }
}

// Power-of-two scale of the fixed-point tally of a unit, and its inverse:
// 2^(50 - E) with bound < 2^E, bound = hits * 2 * m * sum_p |w_p| and m the
// largest |qbar| or incoming |psi| of the unit. psi stays between its
// incoming value and the qbar of the FSRs it crosses (each segment moves it
// toward qbar by the fraction 1 - e^-tau), so every contribution
// sum_p (psi_p - qbar) (1 - e^-tau_p) w_p is at most 2 m sum_p |w_p|.
__device__ __forceinline__ void fixed_scale(float m, float sum_w, int hits, float &scale, float &inv)
{
    const float bound = 2.f * m * sum_w * (float)hits;
    const int E = (int)((__float_as_uint(bound) >> 23) & 0xFFu) - 126; // bound < 2^E (normal bound)
    const int se = max(-126, min(100, MOCGPU_TALLY_BITS - E)); // capped so that weight * scale stays finite
    scale = __uint_as_float((unsigned)(se + 127) << 23);
    inv = __uint_as_float((unsigned)(127 - se) << 23);
}

// Packed FP32 pairs (Blackwell's f32x2 arithmetic): two polar angles' psi
// updates and attenuation arguments in one instruction each, rounded as
// the scalar instructions they replace (MOCGPU_SWEEP_F32X2). Measured: the
// branch batch's sweep 102.4 -> 101.8 ms, the mini-core group sweep about
// 1 % faster.
#ifndef MOCGPU_SWEEP_F32X2
#define MOCGPU_SWEEP_F32X2 1
#endif
__device__ __forceinline__ unsigned long long pk2(float a, float b)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(unsigned long long r, float &a, float &b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Per-unit values a warp needs to sweep one bundle in one direction.
template <typename Real, int NPOL> struct UnitCtx {
    using R2 = typename Pair<Real>::T;
    const Real *ring_len;     // this warp's ring: [ST][CH][32] lengths
    const uint16_t *ring_fsr; // [ST][CH][32] unit-local FSR ids
    const R2 *s_sq;           // (Sigma_t, qbar) per unit FSR
    Real *s_tal;              // FP64 tally copy of this lane
    int *s_hi;                // FP32 fixed-point tally: high words
    unsigned *s_lo;           // and low words (separate arrays: lanes spread over all banks)
    float *tally;             // the solve's FP32 FSR tally (contributions below the fixed-point range)
    const int *lf;            // unit-local -> global FSR ids
    float inv_scale;          // 1 / the unit's fixed-point scale
    Real *psi_in, *psi_out;
    double *cur, *sfl;        // FP64 sweep: the group's currents and surface fluxes
    float *cur32, *sfl32;     // FP32 sweep: their FP32 tallies
    float csgn[2];            // FP32: current of a crossing = csgn[normal] * S (sign and 1 / scale)
    const int (*s_off)[kMaxPolar];
    const int (*s_tgt)[kMaxPolar][2];
    int ny_set;
    Real rsin[NPOL], wt[NPOL];    // wt: polar weights (FP32: times the fixed-point scale)
    unsigned long long rsin2[(NPOL + 1) / 2]; // FP32: rsin of polar pairs, packed
    Real cw[NPOL][2], fwt[NPOL][2]; // current / surface-flux weights
};

// CUR: 0 no coarse tallies; 1 currents and surface fluxes; 2 currents only
// (the batched eigen path: MOCC's surface fluxes only feed the partial-current
// store of CMFD::store_currents, cmfd.cpp:555-666, which the batched engine
// does not run).
//
// One warp sweeps bundle b in one direction (FWD: rows ascending). Per
// segment and polar angle the FP32 path computes psi' = qbar + (psi - qbar)
// E with E = 2^(-tau log2(e) / sin(theta)), and the tally contribution of
// the row as the drop of sum_p w_p psi_p across the segment; that is
// MOCC's psi -= (psi - qbar)(1 - E) and tally += w (psi - qbar)(1 - E)
// (moc_sweeper_kernel.inc.hpp:100-140) summed over the polar angles. The
// FP64 path follows MOCC's form with its table exponential.
//
// The walk is resumable: the unit stages the FSRs of one window of rows at a
// time, and between windows the warp keeps its angular flux, its place in
// the segment ring and its crossing-event cursor in registers. Chunks are
// aligned to absolute rows (chunk k holds rows [k CH, (k + 1) CH)), in both
// directions, so no chunk straddles two windows.
// One state serves both directions (a warp walks one): the direction is a
// template argument of the methods, so the state takes registers once.
template <typename Real, int NPOL, bool GS, int CUR, class SH> struct Walker {
    using R2 = typename Pair<Real>::T;
    static constexpr int CH = SH::rows;
    static constexpr int ST = SH::stages;
    static constexpr bool FIXED = Chunk<Real>::fixed;
    int t, nrows, nch, c, bc_out;
    int64_t row0;
    Real psi[NPOL];
    Real S; // FP32: sum_p w_p psi_p with the current window's scaled weights
    int ev, ev_end;
    int2 ev0, ev1;

    // chunk cc (in sweep order) covers rows [lo, hi)
    template <bool FWD> __device__ __forceinline__ void chunk_rows(int cc, int &lo, int &hi) const
    {
        const int k = FWD ? cc : nch - 1 - cc;
        lo = k * CH;
        hi = min(nrows, lo + CH);
    }
    template <bool FWD>
    __device__ __forceinline__ void issue(const FastView &fv, const UnitCtx<Real, NPOL> &U, int cc, int lane) const
    {
        int lo, hi;
        chunk_rows<FWD>(cc, lo, hi);
        const int nr = hi - lo;
        const int buf = cc % ST;
        const char *gl = (const char *)((const Real *)fv.len + (row0 + lo) * 32);
        char *sl = (char *)(U.ring_len + (size_t)buf * CH * 32);
        const int nl = nr * 32 * (int)sizeof(Real) / 16;
        for (int i = lane; i < nl; i += 32) cp_async16(sl + 16 * i, gl + 16 * i);
        const char *gf = (const char *)(fv.lfsr + (row0 + lo) * 32);
        char *sf = (char *)(U.ring_fsr + (size_t)buf * CH * 32);
        const int nf = nr * 32 * (int)sizeof(uint16_t) / 16;
        for (int i = lane; i < nf; i += 32) cp_async16(sf + 16 * i, gf + 16 * i);
        cp_async_commit();
    }

    template <bool FWD>
    __device__ void begin(const GeomView &g, const FastView &fv, const UnitCtx<Real, NPOL> &U, int b, int lane)
    {
        constexpr int dir = FWD ? 0 : 1;
        t = fv.bundle_track[(size_t)b * 32 + lane];
        const int2 bc = fv.bundle_bc[(size_t)b * 32 + lane];
        nrows = fv.bundle_nrows[b];
        row0 = fv.bundle_row[b];
        nch = (nrows + CH - 1) / CH;
        c = 0;
        const int bc_in = FWD ? bc.x : bc.y;
        bc_out = FWD ? bc.y : bc.x;
        // ST-1 chunks ahead: one commit group per chunk (empty groups past the
        // end keep the count uniform), so waiting until at most ST-1 groups are
        // pending means the chunk about to be swept has landed
        for (int cc = 0; cc < ST - 1; cc++) {
            if (cc < nch) issue<FWD>(fv, U, cc, lane);
            else cp_async_commit();
        }
#pragma unroll
        for (int p = 0; p < NPOL; p++) psi[p] = (t >= 0) ? U.psi_in[U.s_off[dir][p] + bc_in] : (Real)0;
        S = 0;
        if constexpr (FIXED) {
#pragma unroll
            for (int p = 0; p < NPOL; p++) S = fmaf(U.wt[p], psi[p], S); // the same chain as in update()
        }
        ev = ev_end = 0;
        const int2 *evp = FWD ? g.ev_fw : g.ev_bw;
        if (CUR) {
            const int4 e = fv.bundle_ev[(size_t)b * 32 + lane];
            ev = FWD ? e.x : e.z;
            ev_end = FWD ? e.y : e.w;
        }
        const int2 none = make_int2(INT_MAX, 0);
        ev0 = (CUR && ev < ev_end) ? evp[ev] : none;
        ev1 = (CUR && ev + 1 < ev_end) ? evp[ev + 1] : none;
    }

    // the crossing events at row boundary k (the next two live in registers,
    // so a row without an event costs one compare and the load of the event
    // after next has rows of time to arrive)
    template <bool FWD> __device__ __forceinline__ void events(const GeomView &g, const UnitCtx<Real, NPOL> &U, int k)
    {
        const int2 *evp = FWD ? g.ev_fw : g.ev_bw;
        const int2 none = make_int2(INT_MAX, 0);
        while (ev0.x == k) {
            int cd = ev0.y;
            int surf = cd >> 1;
            bool ynorm = cd & 1;
            if constexpr (FIXED) {
                // MOCC's current weight of a crossing (moc_current_worker.hpp:
                // 176-181) is the tally weight w_p with the sign of the
                // direction's x or y cosine, so the current is that sign times
                // S = sum_p w_p psi_p (kept for the tally); FP32 tallies with
                // native float reductions, folded into the FP64 currents when
                // they are normalised
                const float cs = ynorm ? U.csgn[1] : U.csgn[0];
                atomicAdd(U.cur32 + surf, S * (FWD ? cs : -cs));
                if (CUR == 1) {
                    float fc = 0.f;
#pragma unroll
                    for (int p = 0; p < NPOL; p++) fc += psi[p] * (ynorm ? U.fwt[p][1] : U.fwt[p][0]);
                    atomicAdd(U.sfl32 + surf, fc);
                }
            } else {
                Real jc = 0, fc = 0;
#pragma unroll
                for (int p = 0; p < NPOL; p++) {
                    jc += psi[p] * (ynorm ? U.cw[p][1] : U.cw[p][0]);
                    if (CUR == 1) fc += psi[p] * (ynorm ? U.fwt[p][1] : U.fwt[p][0]);
                }
                atomicAdd(U.cur + surf, (double)(FWD ? jc : -jc));
                if (CUR == 1) atomicAdd(U.sfl + surf, (double)fc);
            }
            ev++;
            ev0 = ev1;
            ev1 = (ev + 1 < ev_end) ? evp[ev + 1] : none;
        }
    }

    // FP32 net currents only (CUR == 2): the crossings of a chunk are tallied
    // after its rows. Each row's S before its update (the value a crossing
    // at the row's leading boundary carries) is kept in the row's ring slot,
    // whose length has been read by then; the slots are this lane's own and
    // are refilled only after the warp's closing __syncwarp of the chunk.
    // A row then costs one shared store instead of an event test, and the
    // warp runs the crossing code once per crossing of its busiest lane in
    // the chunk rather than at nearly every row.
    static constexpr bool DEFER = FIXED && CUR == 2;
    template <bool FWD>
    __device__ __forceinline__ void chunk_events(const GeomView &g, const UnitCtx<Real, NPOL> &U, const Real *cl,
                                                 int lo, int hi)
    {
        constexpr int step = FWD ? 32 : -32;
        const int2 *evp = FWD ? g.ev_fw : g.ev_bw;
        const int2 none = make_int2(INT_MAX, 0);
        // forward: boundaries lo .. hi-1 (row k's leading boundary is k);
        // backward: hi .. lo+1 (row k's is k+1), in sweep order
        while (FWD ? ev0.x < hi : (ev0.x > lo && ev0.x != INT_MAX)) {
            const float Sb = cl[(FWD ? ev0.x - lo : hi - ev0.x) * step];
            const int cd = ev0.y;
            const float cs = (cd & 1) ? U.csgn[1] : U.csgn[0];
            atomicAdd(U.cur32 + (cd >> 1), Sb * (FWD ? cs : -cs));
            ev++;
            ev0 = ev1;
            ev1 = (ev + 1 < ev_end) ? evp[ev + 1] : none;
        }
    }

    // Sweeps this direction's chunks whose rows lie in [row_lo, row_hi).
    template <bool FWD>
    __device__ void run(const GeomView &g, const UnitCtx<Real, NPOL> &U, const FastView &fv, int row_lo, int row_hi,
                        int lane)
    {
        // Per row: the factors E (FP32: E = 2^(-tau log2(e) / sin), the
        // transmitted fraction; FP64: 1 - e^-tau from MOCC's table) of a
        // segment in table slot l with Sigma_t sq.x and length L. They do not
        // depend on psi, so a group of rows computes them all before the
        // serial psi updates and tally adds (shared-memory atomics, which
        // later loads cannot pass).
        auto factors = [&](Real L, const R2 &sq, Real (&E)[NPOL]) {
            const Real tau0 = sq.x * L;
#if MOCGPU_SWEEP_F32X2
            if constexpr (FIXED) {
                const unsigned long long t2 = pk2(tau0, tau0);
#pragma unroll
                for (int p = 0; p + 1 < NPOL; p += 2) {
                    float a, b;
                    upk2(mul2(t2, U.rsin2[p / 2]), a, b);
                    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(E[p]) : "f"(a));
                    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(E[p + 1]) : "f"(b));
                }
                if constexpr (NPOL % 2 == 1)
                    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(E[NPOL - 1]) : "f"((float)(tau0 * U.rsin[NPOL - 1])));
                return;
            }
#endif
#pragma unroll
            for (int p = 0; p < NPOL; p++) {
                if constexpr (FIXED) {
                    float e;
                    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"((float)(tau0 * U.rsin[p])));
                    E[p] = e;
                } else {
                    E[p] = atten(tau0, U.rsin[p], g.exp_tab);
                }
            }
        };
        auto update = [&](const R2 &sq, const Real (&E)[NPOL], int l) {
            if constexpr (FIXED) {
                Real S1 = 0;
#if MOCGPU_SWEEP_F32X2
                const unsigned long long q2 = pk2(sq.y, sq.y);
#pragma unroll
                for (int p = 0; p + 1 < NPOL; p += 2) {
                    const unsigned long long ps = fma2(sub2(pk2(psi[p], psi[p + 1]), q2), pk2(E[p], E[p + 1]), q2);
                    upk2(ps, psi[p], psi[p + 1]);
                }
                if constexpr (NPOL % 2 == 1) psi[NPOL - 1] = fmaf(psi[NPOL - 1] - sq.y, E[NPOL - 1], sq.y);
#pragma unroll
                for (int p = 0; p < NPOL; p++) S1 = fmaf(U.wt[p], psi[p], S1);
#else
#pragma unroll
                for (int p = 0; p < NPOL; p++) {
#if MOCGPU_PSI_FMA2
                    psi[p] = fmaf(psi[p], E[p], fmaf(-sq.y, E[p], sq.y));
#else
                    psi[p] = fmaf(psi[p] - sq.y, E[p], sq.y);
#endif
                    S1 = fmaf(U.wt[p], psi[p], S1);
                }
#endif
                tally_fixed(U.s_hi, U.s_lo, U.tally, U.lf, U.inv_scale, l, S - S1);
                S = S1;
            } else {
                Real acc = 0;
#pragma unroll
                for (int p = 0; p < NPOL; p++) {
                    Real d = (psi[p] - sq.y) * E[p];
                    psi[p] -= d;
                    acc += d * U.wt[p];
                }
                tally_add(U.s_tal, l, acc);
            }
        };

        while (c < nch) {
            int lo, hi;
            chunk_rows<FWD>(c, lo, hi);
            if (FWD ? lo >= row_hi : lo < row_lo) break; // the chunk belongs to a later window
            if (c + ST - 1 < nch) issue<FWD>(fv, U, c + ST - 1, lane);
            else cp_async_commit();
            cp_async_wait<ST - 1>();
            __syncwarp();
            const int nr = hi - lo;
            // rows of this chunk in sweep order: FWD from the first, else from the last
            const Real *cl = U.ring_len + (size_t)(c % ST) * CH * 32 + (FWD ? 0 : (nr - 1) * 32) + lane;
            const uint16_t *cf = U.ring_fsr + (size_t)(c % ST) * CH * 32 + (FWD ? 0 : (nr - 1) * 32) + lane;
            constexpr int step = FWD ? 32 : -32;
            // UR rows per step: the loads and gathers of the rows issue back
            // to back; only the psi recurrence that follows is serial.
            constexpr int UR = SH::unroll;
            int k = 0;
            for (; k + UR <= nr; k += UR) {
                Real L[UR];
                int l[UR];
                R2 sq[UR];
                Real E[UR][NPOL];
#pragma unroll
                for (int v = 0; v < UR; v++) {
                    L[v] = cl[(k + v) * step];
                    l[v] = cf[(k + v) * step];
                }
#pragma unroll
                for (int v = 0; v < UR; v++) sq[v] = U.s_sq[l[v]];
#pragma unroll
                for (int v = 0; v < UR; v++) factors(L[v], sq[v], E[v]);
#pragma unroll
                for (int v = 0; v < UR; v++) {
                    if constexpr (DEFER) const_cast<Real *>(cl)[(k + v) * step] = S;
                    else if (CUR && t >= 0) events<FWD>(g, U, FWD ? lo + k + v : hi - (k + v));
                    update(sq[v], E[v], l[v]);
                }
            }
            for (; k < nr; k++) {
                const int l = cf[k * step];
                const R2 sq = U.s_sq[l];
                Real E[NPOL];
                factors(cl[k * step], sq, E);
                if constexpr (DEFER) const_cast<Real *>(cl)[k * step] = S;
                else if (CUR && t >= 0) events<FWD>(g, U, FWD ? lo + k : hi - k);
                update(sq, E, l);
            }
            if constexpr (DEFER)
                if (t >= 0) chunk_events<FWD>(g, U, cl, lo, hi);
            __syncwarp();
            c++;
        }
    }

    // After the last row: the crossing at the track's end and the outgoing
    // angular flux (Gauss-Seidel: straight into the reflected angle's
    // incoming entry).
    template <bool FWD> __device__ void finish(const GeomView &g, const UnitCtx<Real, NPOL> &U)
    {
        constexpr int dir = FWD ? 0 : 1;
        if (t < 0) return;
        if (CUR) events<FWD>(g, U, FWD ? nrows : 0);
#pragma unroll
        for (int p = 0; p < NPOL; p++) {
            if (GS) {
                // reflected angle's entry, or zero on a vacuum face (-1 - offset)
                const int tgt = U.s_tgt[dir][p][bc_out < U.ny_set ? 0 : 1];
                U.psi_in[(tgt >= 0 ? tgt : -1 - tgt) + bc_out] = tgt >= 0 ? psi[p] : (Real)0;
            } else {
                U.psi_out[U.s_off[dir][p] + bc_out] = psi[p];
            }
        }
    }
};

// One FSR table in shared memory: the (Sigma_t, qbar) pairs of a window's
// FSRs and their tally (FP32: fixed-point high and low words; FP64: the
// tally copies), slot n_local being the padding slot.
template <typename Real> struct Table {
    using R2 = typename Pair<Real>::T;
    R2 *sq;
    int *hi;       // FP32
    unsigned *lo;  // FP32
    Real *tal;     // FP64: [TC][slots]
    __device__ void place(unsigned char *base, int slots)
    {
        sq = reinterpret_cast<R2 *>(base);
        hi = reinterpret_cast<int *>(sq + slots);
        lo = reinterpret_cast<unsigned *>(hi + slots);
        tal = reinterpret_cast<Real *>(sq + slots);
    }
};

// WIN: the layout may have units of several row windows (the single-solve
// kernel); without it (the batched kernel, whose geometries are laid out in
// whole units) the window loop folds away and takes no registers.
template <typename Real, int NPOL, bool GS, int CUR, class SH, bool WIN>
__device__ __forceinline__ void sweep_unit(const GeomView &g, const FastView &fv, const StateView &st, int group,
                                           int wu, unsigned char *smem_raw)
{
    using R2 = typename Pair<Real>::T;
    constexpr int CH = SH::rows;
    constexpr int ST = SH::stages;
    constexpr int TC = Chunk<Real>::tally_copies;
    constexpr bool FIXED = Chunk<Real>::fixed;
    const WorkUnitDev u = fv.wu[wu];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int K = WIN ? u.n_win : 1, slots = fv.table_slots;
    // [warp rings][table A][table B]: A holds the window the forward warps
    // sweep, B the one the backward warps sweep (A serves both when they are
    // the same window)
    unsigned char *ring = smem_raw + (size_t)warp * ring_bytes<Real, SH>();
    unsigned char *tables = smem_raw + (size_t)nwarps * ring_bytes<Real, SH>();
    // table pointers are recomputed where they are needed (fewer registers
    // live across the sweep)
    auto table = [&](int which) {
        Table<Real> T;
        T.place(tables + (size_t)which * slots * fsr_slot_bytes<Real>(), slots);
        return T;
    };

    UnitCtx<Real, NPOL> U;
    U.ring_len = reinterpret_cast<const Real *>(ring);
    U.ring_fsr = reinterpret_cast<const uint16_t *>(ring + ST * CH * 32 * sizeof(Real));
    U.psi_in = (Real *)st.psi_in + (size_t)group * g.bc_per_group;
    U.psi_out = (Real *)st.psi_out;
    U.cur = st.cur + (size_t)group * g.n_surf;
    U.sfl = st.sflux + (size_t)group * g.n_surf;
    U.cur32 = st.cur32 + (size_t)(blockIdx.x % kCurCopies) * g.n_surf;
    U.sfl32 = st.sfl32 + (size_t)(blockIdx.x % kCurCopies) * g.n_surf;
    U.tally = (float *)st.tally;
    U.ny_set = g.set_ny[u.set];

    // per unit: boundary-flux offsets of every (direction, polar) angle and
    // the reflected angles' incoming offsets for the Gauss-Seidel write-through
    // (stored as -1 - offset where the face is vacuum: the entry is zeroed,
    // as BoundaryCondition::update does, boundary_condition.cpp:155-191)
    __shared__ int s_off[2][kMaxPolar], s_tgt[2][kMaxPolar][2];
    __shared__ unsigned s_mbits; // largest |qbar| or incoming |psi| staged so far (float bits)
    U.s_off = s_off;
    U.s_tgt = s_tgt;
    if (threadIdx.x < 2 * NPOL) {
        const int dir = threadIdx.x / NPOL, p = threadIdx.x % NPOL;
        const SetPolar sp = g.sp[u.set * NPOL + p];
        const int a = dir == 0 ? sp.ang_fwd : sp.ang_bwd;
        s_off[dir][p] = g.bc_off[a];
        if (GS) {
            for (int n = 0; n < 2; n++) {
                const int base = g.wt_tgt[3 * g.n_ang + a * 2 + n];
                s_tgt[dir][p][n] = g.wt_tgt[a * 2 + n] >= 0 ? base : -1 - base;
            }
        }
    }
    if (FIXED && threadIdx.x == 0) s_mbits = 0u;
#pragma unroll
    for (int p = 0; p < NPOL; p++) {
        const SetPolar sp = g.sp[u.set * NPOL + p];
        U.rsin[p] = polar_factor<Real>(sp.rsin);
        U.wt[p] = (Real)sp.wt;
        if constexpr (FIXED) {
            if (p % 2 == 1) U.rsin2[p / 2] = pk2((float)U.rsin[p - 1], (float)U.rsin[p]);
        }
        if (CUR) {
            U.cw[p][0] = (Real)sp.cw[0];
            U.cw[p][1] = (Real)sp.cw[1];
            U.fwt[p][0] = (Real)sp.fw[0];
            U.fwt[p][1] = (Real)sp.fw[1];
        }
    }
    __syncthreads();

    const Real *sigt = (const Real *)st.sigt;
    const Real *qbar = (const Real *)st.qbar;
    // stages window w into table T: (Sigma_t, qbar) of its FSRs, zero
    // tallies, the zero padding slot; returns the largest |qbar| (float bits)
    auto stage = [&](Table<Real> T, int w) -> unsigned {
        const int2 wi = fv.win[w]; // (first entry in local_fsr, FSRs)
        const int *lf = fv.local_fsr + wi.x;
        unsigned mb = 0u; // float bits of a non-negative value order like the integers
        // four FSRs per thread in flight, so the dependent loads (local id,
        // then Sigma_t and qbar) overlap
        for (int i0 = threadIdx.x; i0 < wi.y; i0 += 4 * blockDim.x) {
            int gl[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = i0 + j * blockDim.x;
                gl[j] = (i < wi.y) ? lf[i] : -1;
            }
            Real sg[4], qq[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                sg[j] = gl[j] >= 0 ? sigt[gl[j]] : (Real)0;
                qq[j] = gl[j] >= 0 ? qbar[gl[j]] : (Real)0;
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = i0 + j * blockDim.x;
                if (i >= wi.y) break;
                T.sq[i] = R2{sg[j], qq[j]};
                if constexpr (FIXED) {
                    mb = max(mb, __float_as_uint(fabsf((float)qq[j])));
                    T.hi[i] = 0;
                    T.lo[i] = 0u;
                } else {
#pragma unroll
                    for (int cc = 0; cc < TC; cc++) T.tal[(size_t)cc * slots + i] = (Real)0;
                }
            }
        }
        // padding entries point at the slot after the window's FSRs, which
        // holds Sigma_t = qbar = 0: a padding row leaves psi unchanged bit
        // for bit and adds nothing
        if (threadIdx.x == 0) T.sq[wi.y] = R2{(Real)0, (Real)0};
        return mb;
    };
    // adds table T's tally (window w) to the solve's FSR tally
    auto flush = [&](Table<Real> T, int w, float inv) {
        const int2 wi = fv.win[w];
        const int *lf = fv.local_fsr + wi.x;
        Real *tally = (Real *)st.tally;
        for (int i = threadIdx.x; i < wi.y; i += blockDim.x) {
            Real v;
            if constexpr (FIXED) {
                const long long x = (long long)T.hi[i] * (1ll << 20) + (long long)T.lo[i];
                v = (Real)(__ll2float_rn(x) * inv);
            } else {
                v = T.tal[i];
#pragma unroll
                for (int cc = 1; cc < TC; cc++) v += T.tal[(size_t)cc * slots + i];
            }
            if (v != (Real)0) atomicAdd(tally + lf[i], v);
        }
    };

    // this warp's task: bundle b, forward (even warps) or backward (odd);
    // a unit has at most as many bundles as a CTA has warp pairs
    const bool has_task = warp < 2 * u.n_bundles;
    const bool fwd = (warp & 1) == 0;
    const int b = u.bundle_begin + (warp >> 1);
    Walker<Real, NPOL, GS, CUR, SH> w;
    float scale = 1.f, inv_scale = 1.f;
    for (int j = 0; j < K; j++) {
        const int wa = u.win_begin + j, wbk = u.win_begin + K - 1 - j;
        const bool same = !WIN || wa == wbk;
        unsigned mb = stage(table(0), wa);
        if (!same) mb = max(mb, stage(table(1), wbk));
        if constexpr (FIXED) {
            if (j == 0) {
                // incoming angular fluxes of every lane, direction and polar angle
                for (int i = threadIdx.x; i < u.n_bundles * 64; i += blockDim.x) {
                    const size_t bl = (size_t)(u.bundle_begin + (i >> 6)) * 32 + (i & 31);
                    const int dir = (i >> 5) & 1;
                    if (fv.bundle_track[bl] < 0) continue;
                    const int2 bc = fv.bundle_bc[bl];
                    const int bc_in = dir == 0 ? bc.x : bc.y;
#pragma unroll
                    for (int p = 0; p < NPOL; p++)
                        mb = max(mb, __float_as_uint(fabsf((float)U.psi_in[s_off[dir][p] + bc_in])));
                }
            }
            mb = __reduce_max_sync(0xffffffffu, mb);
            if (lane == 0 && mb) atomicMax(&s_mbits, mb);
        }
        __syncthreads();
        if constexpr (FIXED) {
            // Power-of-two scale of this window's fixed-point tally from the
            // largest qbar or incoming psi staged so far, which bounds psi in
            // the rows swept up to here; the running sums S change scale
            // exactly with it.
            const unsigned mbits = s_mbits;
            if (mbits >= 0x7F800000u && threadIdx.x == 0) atomicOr(st.status, (unsigned)DEV_NAN); // inf or NaN
            float sum_w = 0.f, w0[NPOL];
#pragma unroll
            for (int p = 0; p < NPOL; p++) {
                w0[p] = (float)g.sp[u.set * NPOL + p].wt;
                sum_w += fabsf(w0[p]);
            }
            float sc, inv;
            fixed_scale(__uint_as_float(mbits), sum_w, fv.max_hits, sc, inv);
            const float ratio = sc * inv_scale;
            scale = sc;
            inv_scale = inv;
#pragma unroll
            for (int p = 0; p < NPOL; p++) U.wt[p] = w0[p] * scale;
            U.inv_scale = inv_scale;
            if (CUR) {
                const SetPolar sp0 = g.sp[u.set * NPOL];
                U.csgn[0] = copysignf(inv_scale, (float)sp0.cw[0]);
                U.csgn[1] = copysignf(inv_scale, (float)sp0.cw[1]);
            }
            if (j > 0 && has_task) w.S *= ratio;
        }
        if (has_task) {
            const Table<Real> T = table((fwd || same) ? 0 : 1);
            const int2 wi = fv.win[fwd ? wa : wbk];
            U.s_sq = T.sq;
            U.s_hi = T.hi;
            U.s_lo = T.lo;
            U.s_tal = T.tal + (size_t)(lane % TC) * slots;
            U.lf = fv.local_fsr + wi.x;
            const int wr = (WIN && K > 1) ? fv.window_rows : INT_MAX / 2;
            if (fwd) {
                if (j == 0) w.template begin<true>(g, fv, U, b, lane);
                w.template run<true>(g, U, fv, j * wr, (j + 1) * wr, lane);
                if (j == K - 1) w.template finish<true>(g, U);
            } else {
                if (j == 0) w.template begin<false>(g, fv, U, b, lane);
                w.template run<false>(g, U, fv, (K - 1 - j) * wr, (K - j) * wr, lane);
                if (j == K - 1) w.template finish<false>(g, U);
            }
        }
        __syncthreads();
        flush(table(0), wa, inv_scale);
        if (!same) flush(table(1), wbk, inv_scale);
        if (j + 1 < K) __syncthreads(); // the next window's staging overwrites the tables
    }
}

void note_launch_external();

template <typename Real, int NPOL, bool GS, int CUR>
__global__ void k_sweep_fast(GeomView g, FastView fv, StateView st, int group, int wu0)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    sweep_unit<Real, NPOL, GS, CUR, DefaultShape, true>(g, fv, st, group, wu0 + blockIdx.x, smem_raw);
}

// Persistent batched sweep: a fixed grid walks the (solve slot, work unit)
// list of every active solve, largest units first. Each CTA starts on item
// blockIdx.x and then takes the next untaken item from a counter (zeroed
// once per graph replay), so CTAs that drew short units take more of them
// and the launch ends with little tail.
template <typename Real, int NPOL, int CUR, class SH>
__global__ void MOCGPU_SWEEP_BOUNDS kb_sweep_fast(BatchViews b, const int2 *items, const int *n_items, int group,
                                                  int *counter)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_next;
    const int n = *n_items;
    int it = blockIdx.x;
    while (it < n) {
        const int2 item = items[it];
        // solves that ended in an earlier replay are frozen (uniform per CTA)
        if (b.sv[item.x].red[RED_DONE] == 0.0)
            sweep_unit<Real, NPOL, true, CUR, SH, false>(b.gv[item.x], b.fv[item.x], b.sv[item.x], group, item.y,
                                                         smem_raw);
        if (threadIdx.x == 0) s_next = (int)gridDim.x + atomicAdd(counter, 1);
        __syncthreads(); // also: the next unit may overwrite this one's shared data
        it = s_next;
    }
}

template <typename Real, class SH> static size_t batched_smem(int bundles_per_unit, int max_local)
{
    return (size_t)(2 * bundles_per_unit) * ring_bytes<Real, SH>() + (size_t)max_local * fsr_slot_bytes<Real>();
}

// The batched engine runs the Gauss-Seidel boundary update only, so the
// batched kernel is built for it alone.
template <typename Real, class SH> static void prepare_batched_shape(int pol, int bundles_per_unit, int max_local)
{
    const size_t smem = batched_smem<Real, SH>(bundles_per_unit, max_local);
    switch (pol) {
#define MOCGPU_P(NP)                                                                                                   \
    case NP:                                                                                                           \
        ensure_smem_limit((const void *)kb_sweep_fast<Real, NP, 0, SH>, smem);                                        \
        ensure_smem_limit((const void *)kb_sweep_fast<Real, NP, 1, SH>, smem);                                        \
        ensure_smem_limit((const void *)kb_sweep_fast<Real, NP, 2, SH>, smem);                                        \
        return;
        MOCGPU_P(1)
        MOCGPU_P(2)
        MOCGPU_P(3)
        MOCGPU_P(4)
#undef MOCGPU_P
    }
    throw Error(1, "unsupported number of polar angles per track set");
}

template <typename Real, int NPOL, int CUR, class SH>
static void launch_batched(const BatchViews &b, const int2 *items, const int *n_items, int max_items, int group,
                           int bundles_per_unit, int max_local, int *counter, cudaStream_t s)
{
    auto k = kb_sweep_fast<Real, NPOL, CUR, SH>;
    const int nwarps = 2 * bundles_per_unit;
    const size_t smem = batched_smem<Real, SH>(bundles_per_unit, max_local);
    ensure_smem_limit((const void *)k, smem);
    int per_sm = 1;
    MOCGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 32 * nwarps, smem));
    int dev = 0, sms = 152;
    MOCGPU_CUDA(cudaGetDevice(&dev));
    MOCGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int grid = std::max(1, std::min(max_items, sms * std::max(1, per_sm)));
    k<<<grid, 32 * nwarps, smem, s>>>(b, items, n_items, group, counter);
}

// cur: 0 no coarse tallies, 1 net currents and surface fluxes, 2 net
// currents only (all the CMFD operator reads)
template <typename Real, class SH>
static void launch_batched_shape(const BatchViews &b, const int2 *items, const int *n_items, int max_items, int group,
                                 int cur, int pol, int bundles_per_unit, int max_local, int *counter, cudaStream_t s)
{
    switch (pol) {
#define MOCGPU_B(NP)                                                                                                   \
    case NP:                                                                                                           \
        if (cur == 2) launch_batched<Real, NP, 2, SH>(b, items, n_items, max_items, group, bundles_per_unit,          \
                                                      max_local, counter, s);                                          \
        else if (cur == 1) launch_batched<Real, NP, 1, SH>(b, items, n_items, max_items, group, bundles_per_unit,     \
                                                           max_local, counter, s);                                     \
        else launch_batched<Real, NP, 0, SH>(b, items, n_items, max_items, group, bundles_per_unit, max_local,        \
                                             counter, s);                                                              \
        return;
        MOCGPU_B(1)
        MOCGPU_B(2)
        MOCGPU_B(3)
        MOCGPU_B(4)
#undef MOCGPU_B
    }
    throw Error(1, "unsupported number of polar angles per track set");
}

// FP32 batched sweep in shapes 1-2 (sweep_fast_shapes_a.cu) and 3-4
// (sweep_fast_shapes_b.cu); false when `shape` is not one of theirs.
bool prepare_b_sweep_shapes_a(int shape, int pol, int bundles_per_unit, int max_local);
bool prepare_b_sweep_shapes_b(int shape, int pol, int bundles_per_unit, int max_local);
bool launch_b_sweep_shapes_a(int shape, const BatchViews &b, const int2 *items, const int *n_items, int max_items,
                             int group, int cur, int pol, int bundles_per_unit, int max_local, int *counter,
                             cudaStream_t s);
bool launch_b_sweep_shapes_b(int shape, const BatchViews &b, const int2 *items, const int *n_items, int max_items,
                             int group, int cur, int pol, int bundles_per_unit, int max_local, int *counter,
                             cudaStream_t s);

} // namespace mocgpu
