// Bundled work-unit MoC sweep (the sweep of moc_sweeper_kernel.inc.hpp:36-180,
// rearranged for the GPU).
//
// One CTA per work unit. The unit's FSR cross sections and sources are staged
// into shared memory as (Sigma_t, qbar) pairs and the unit's FSR tally lives
// in shared memory; one warp sweeps one bundle of 32 tracks, one track per
// lane, all polar angles of the azimuth in registers. Segment rows are read
// 32-wide and coalesced. With `split` the forward and the backward pass of a
// bundle run on two warps; otherwise one lane does both in the same loop.
// After the bundles, the unit's tally is added to the global FSR tally with
// one atomic per touched FSR.
#include "kernels.cuh"

namespace mocgpu {

__device__ __forceinline__ double att_fast(double tau, const double *tab)
{
    double v = -tau;
    if (v < -10.0 || v > 0.0) return 1.0 - exp(v);
    const double rspace = 1000.0, space = 1.0e-3; // 10000 intervals on [-10, 0]
    int i = (int)((v + 10.0) * rspace);
    if (i >= kExpN) i = kExpN - 1;
    v -= space * i - 10.0;
    double d0 = __ldg(tab + i), d1 = __ldg(tab + i + 1);
    return 1.0 - (d0 + (d1 - d0) * v * rspace);
}
__device__ __forceinline__ float att_fast(float tau, const double *)
{
    if (tau < 0.015625f) return tau * (1.0f - tau * (0.5f - tau * (0.16666667f - tau * 0.041666668f)));
    return 1.0f - __expf(-tau);
}

template <typename Real> struct Pair;
template <> struct Pair<float> {
    using T = float2;
};
template <> struct Pair<double> {
    using T = double2;
};

template <typename Real, int NPOL, bool GS, bool CUR, bool SPLIT>
__global__ void k_sweep_fast(GeomView g, FastView fv, StateView st, int group, int wu0)
{
    using R2 = typename Pair<Real>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const WorkUnitDev u = fv.wu[wu0 + blockIdx.x];
    R2 *s_sq = reinterpret_cast<R2 *>(smem_raw);
    Real *s_tal = reinterpret_cast<Real *>(s_sq + fv.max_local);

    const Real *sigt = (const Real *)st.sigt;
    const Real *qbar = (const Real *)st.qbar;
    for (int i = threadIdx.x; i < u.n_local; i += blockDim.x) {
        int gl = fv.local_fsr[u.fsr_begin + i];
        s_sq[i] = R2{sigt[gl], qbar[gl]};
        s_tal[i] = (Real)0;
    }
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int ntasks = SPLIT ? 2 * u.n_bundles : u.n_bundles;
    const Real *lenp = (const Real *)fv.len;
    Real *psi_in = (Real *)st.psi_in + (size_t)group * g.bc_per_group;
    Real *psi_out = (Real *)st.psi_out;
    const int ny_set = g.set_ny[u.set];

    Real rsin[NPOL], wt[NPOL];
    int af[NPOL], ab[NPOL];
    double cw[NPOL][2], fwt[NPOL][2];
#pragma unroll
    for (int p = 0; p < NPOL; p++) {
        const SetPolar sp = g.sp[u.set * NPOL + p];
        rsin[p] = (Real)sp.rsin;
        wt[p] = (Real)sp.wt;
        af[p] = sp.ang_fwd;
        ab[p] = sp.ang_bwd;
        if (CUR) {
            cw[p][0] = sp.cw[0];
            cw[p][1] = sp.cw[1];
            fwt[p][0] = sp.fw[0];
            fwt[p][1] = sp.fw[1];
        }
    }
    double *cur = st.cur + (size_t)group * g.n_surf;
    double *sfl = st.sflux + (size_t)group * g.n_surf;

    for (int task = warp; task < ntasks; task += nwarps) {
        const int b = u.bundle_begin + (SPLIT ? (task >> 1) : task);
        const bool do_fwd = SPLIT ? ((task & 1) == 0) : true;
        const bool do_bwd = SPLIT ? ((task & 1) == 1) : true;
        const int t = fv.bundle_track[(size_t)b * 32 + lane];
        const int nrows = fv.bundle_nrows[b];
        const int64_t base = fv.bundle_row[b] * 32 + lane;
        int n = 0, bc0 = 0, bc1 = 0;
        Real pf[NPOL], pb[NPOL];
        if (t >= 0) {
            n = (int)(g.seg_begin[t + 1] - g.seg_begin[t]);
            bc0 = g.trk_bc0[t];
            bc1 = g.trk_bc1[t];
        }
#pragma unroll
        for (int p = 0; p < NPOL; p++) {
            pf[p] = (t >= 0 && do_fwd) ? psi_in[g.bc_off[af[p]] + bc0] : (Real)0;
            pb[p] = (t >= 0 && do_bwd) ? psi_in[g.bc_off[ab[p]] + bc1] : (Real)0;
        }
        int evf = 0, evf_end = 0, evb = 0, evb_end = 0;
        if (CUR && t >= 0) {
            if (do_fwd) {
                evf = g.ev_fw_begin[t];
                evf_end = g.ev_fw_begin[t + 1];
            }
            if (do_bwd) {
                evb = g.ev_bw_begin[t];
                evb_end = g.ev_bw_begin[t + 1];
            }
        }
        auto events = [&](const int *pt, const int *code, int &ev, int ev_end, int k, double sign, const Real *psi) {
            while (ev < ev_end && pt[ev] == k) {
                int c = code[ev];
                int surf = c >> 1;
                bool ynorm = c & 1;
                double jc = 0.0, fc = 0.0;
#pragma unroll
                for (int p = 0; p < NPOL; p++) {
                    jc += (double)psi[p] * (ynorm ? cw[p][1] : cw[p][0]);
                    fc += (double)psi[p] * (ynorm ? fwt[p][1] : fwt[p][0]);
                }
                atomicAdd(cur + surf, sign * jc);
                atomicAdd(sfl + surf, fc);
                ev++;
            }
        };

        // software pipeline: rows for step r+1 are loaded while step r computes
        Real Lf = 0, Lb = 0;
        int lf = 0, lb = 0;
        if (nrows > 0) {
            if (do_fwd) {
                Lf = lenp[base];
                lf = fv.lfsr[base];
            }
            if (do_bwd) {
                Lb = lenp[base + (int64_t)(nrows - 1) * 32];
                lb = fv.lfsr[base + (int64_t)(nrows - 1) * 32];
            }
        }
        for (int r = 0; r < nrows; r++) {
            Real nLf = 0, nLb = 0;
            int nlf = 0, nlb = 0;
            if (r + 1 < nrows) {
                if (do_fwd) {
                    nLf = lenp[base + (int64_t)(r + 1) * 32];
                    nlf = fv.lfsr[base + (int64_t)(r + 1) * 32];
                }
                if (do_bwd) {
                    nLb = lenp[base + (int64_t)(nrows - 2 - r) * 32];
                    nlb = fv.lfsr[base + (int64_t)(nrows - 2 - r) * 32];
                }
            }
            if (do_fwd) {
                if (CUR && t >= 0) events(g.ev_fw_pt, g.ev_fw_code, evf, evf_end, r, 1.0, pf);
                const R2 sq = s_sq[lf];
                const Real tau0 = sq.x * Lf;
                Real acc = 0;
#pragma unroll
                for (int p = 0; p < NPOL; p++) {
                    Real e = att_fast(tau0 * rsin[p], g.exp_tab);
                    Real d = (pf[p] - sq.y) * e;
                    pf[p] -= d;
                    acc += d * wt[p];
                }
                if (Lf > (Real)0) atomicAdd(s_tal + lf, acc);
            }
            if (do_bwd) {
                const int row = nrows - 1 - r;
                if (CUR && t >= 0) events(g.ev_bw_pt, g.ev_bw_code, evb, evb_end, row + 1, -1.0, pb);
                const R2 sq = s_sq[lb];
                const Real tau0 = sq.x * Lb;
                Real acc = 0;
#pragma unroll
                for (int p = 0; p < NPOL; p++) {
                    Real e = att_fast(tau0 * rsin[p], g.exp_tab);
                    Real d = (pb[p] - sq.y) * e;
                    pb[p] -= d;
                    acc += d * wt[p];
                }
                if (Lb > (Real)0) atomicAdd(s_tal + lb, acc);
            }
            Lf = nLf;
            lf = nlf;
            Lb = nLb;
            lb = nlb;
        }
        if (t >= 0) {
            if (CUR) {
                if (do_fwd) events(g.ev_fw_pt, g.ev_fw_code, evf, evf_end, nrows, 1.0, pf);
                if (do_bwd) events(g.ev_bw_pt, g.ev_bw_code, evb, evb_end, 0, -1.0, pb);
            }
            (void)n;
#pragma unroll
            for (int p = 0; p < NPOL; p++) {
                if (do_fwd) {
                    if (GS) {
                        int tgt = g.wt_tgt[af[p] * 2 + (bc1 < ny_set ? 0 : 1)];
                        if (tgt >= 0) psi_in[tgt + bc1] = pf[p];
                    } else {
                        psi_out[g.bc_off[af[p]] + bc1] = pf[p];
                    }
                }
                if (do_bwd) {
                    if (GS) {
                        int tgt = g.wt_tgt[ab[p] * 2 + (bc0 < ny_set ? 0 : 1)];
                        if (tgt >= 0) psi_in[tgt + bc0] = pb[p];
                    } else {
                        psi_out[g.bc_off[ab[p]] + bc0] = pb[p];
                    }
                }
            }
        }
    }
    __syncthreads();
    Real *tally = (Real *)st.tally;
    for (int i = threadIdx.x; i < u.n_local; i += blockDim.x) {
        Real v = s_tal[i];
        if (v != (Real)0) atomicAdd(tally + fv.local_fsr[u.fsr_begin + i], v);
    }
}

template <typename Real> size_t fast_sweep_smem(const FastView &fv)
{
    return (size_t)fv.max_local * (3 * sizeof(Real));
}
template size_t fast_sweep_smem<float>(const FastView &);
template size_t fast_sweep_smem<double>(const FastView &);

template <typename Real, int NPOL, bool GS, bool CUR, bool SPLIT>
static void launch_one(const GeomView &g, const FastView &fv, const StateView &st, int group, int wu0, int wu1,
                       cudaStream_t s)
{
    auto k = k_sweep_fast<Real, NPOL, GS, CUR, SPLIT>;
    size_t smem = fast_sweep_smem<Real>(fv);
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        MOCGPU_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = smem;
    }
    int threads = 32 * fv.bundles_per_unit * (SPLIT ? 2 : 1);
    k<<<wu1 - wu0, threads, smem, s>>>(g, fv, st, group, wu0);
}

template <typename Real, int NPOL>
static void launch_np(const GeomView &g, const FastView &fv, const StateView &st, int group, int wu0, int wu1, bool gs,
                      bool cur, cudaStream_t s)
{
#define MOCGPU_FAST_CASE(GS_, CUR_, SPLIT_)                                                                           \
    if (gs == GS_ && cur == CUR_ && (fv.split != 0) == SPLIT_) {                                                     \
        launch_one<Real, NPOL, GS_, CUR_, SPLIT_>(g, fv, st, group, wu0, wu1, s);                                     \
        return;                                                                                                      \
    }
    MOCGPU_FAST_CASE(true, false, true)
    MOCGPU_FAST_CASE(true, true, true)
    MOCGPU_FAST_CASE(false, false, true)
    MOCGPU_FAST_CASE(false, true, true)
    MOCGPU_FAST_CASE(true, false, false)
    MOCGPU_FAST_CASE(true, true, false)
    MOCGPU_FAST_CASE(false, false, false)
    MOCGPU_FAST_CASE(false, true, false)
#undef MOCGPU_FAST_CASE
}

void note_launch_external();

template <typename Real>
void launch_sweep_fast(const GeomView &g, const FastView &fv, const StateView &st, int group, int wu0, int wu1,
                       bool gs, bool cur, cudaStream_t s)
{
    if (wu1 <= wu0) return;
    note_launch_external();
    switch (g.pol) {
    case 1: launch_np<Real, 1>(g, fv, st, group, wu0, wu1, gs, cur, s); break;
    case 2: launch_np<Real, 2>(g, fv, st, group, wu0, wu1, gs, cur, s); break;
    case 3: launch_np<Real, 3>(g, fv, st, group, wu0, wu1, gs, cur, s); break;
    case 4: launch_np<Real, 4>(g, fv, st, group, wu0, wu1, gs, cur, s); break;
    default: throw Error(1, "unsupported number of polar angles per track set");
    }
}
template void launch_sweep_fast<float>(const GeomView &, const FastView &, const StateView &, int, int, int, bool, bool,
                                       cudaStream_t);
template void launch_sweep_fast<double>(const GeomView &, const FastView &, const StateView &, int, int, int, bool,
                                        bool, cudaStream_t);

} // namespace mocgpu
