// Kernels for the MoC transport sweep and the CMFD-accelerated power
// iteration around it. Each kernel cites the MOCC routine whose arithmetic
// it follows; the structure (one launch per pass over HBM-resident arrays)
// is this project's own.
#include <atomic>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>

#include "kernels.cuh"

namespace mocgpu {

constexpr double kFpi = 4.0 * 3.1415926535897932;

// Number of kernels this library has launched (all streams, all handles).
static std::atomic<int64_t> g_launches{0};
static inline void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
int64_t launch_count() { return g_launches.load(); }
void note_launch_external() { note_launch(); }
void note_launches(int64_t n) { g_launches += n; }
static std::atomic<int64_t> g_h2d{0}, g_d2h{0};
void note_copy_bytes(cudaMemcpyKind kind, size_t bytes)
{
    if (kind == cudaMemcpyHostToDevice) g_h2d += (int64_t)bytes;
    else if (kind == cudaMemcpyDeviceToHost) g_d2h += (int64_t)bytes;
}
void copy_bytes(int64_t *h2d, int64_t *d2h)
{
    *h2d = g_h2d.load();
    *d2h = g_d2h.load();
}

static std::atomic<int64_t> g_alloc_fault{-1};
void set_alloc_fault(int64_t after) { g_alloc_fault.store(after); }
bool alloc_fault_due()
{
    int64_t v = g_alloc_fault.load();
    while (v >= 0) {
        if (g_alloc_fault.compare_exchange_weak(v, v - 1)) return v == 0;
    }
    return false;
}

// Function attributes are per device: remember what was set for each
// (kernel, device, attribute) and raise it only when a launch needs more.
void raise_func_attr(const void *kernel, cudaFuncAttribute attr, int value)
{
    static std::mutex mu;
    static std::map<std::tuple<const void *, int, int>, int> set;
    int dev = 0;
    MOCGPU_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    int &cur = set[std::make_tuple(kernel, dev, (int)attr)];
    if (value > cur) {
        MOCGPU_CUDA(cudaFuncSetAttribute(kernel, attr, value));
        cur = value;
    }
}
void ensure_smem_limit(const void *kernel, size_t bytes)
{
    if (bytes > 48 * 1024) raise_func_attr(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// ---------------------------------------------------------------------------
__global__ void k_fill(double *p, double v, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}
template <typename Real> __global__ void k_fill_real(Real *p, double v, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (Real)v;
}

static int grid_for(int64_t n, int block, int cap = 152 * 16)
{
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

void launch_fill(double *p, double v, int64_t n, cudaStream_t s)
{
    if (n > 0) { note_launch(); k_fill<<<grid_for(n, 256), 256, 0, s>>>(p, v, n); }
}
template <typename Real> void launch_fill_real(Real *p, double v, int64_t n, cudaStream_t s)
{
    if (n > 0) { note_launch(); k_fill_real<Real><<<grid_for(n, 256), 256, 0, s>>>(p, v, n); }
}
template void launch_fill_real<float>(float *, double, int64_t, cudaStream_t);
template void launch_fill_real<double>(double *, double, int64_t, cudaStream_t);

// ---------------------------------------------------------------------------
// fs_r = sum_g (1/k) nuSigma_f,g phi_g,r   (transport_sweeper.cpp:119-134)
__global__ void k_fission_source(GeomView g, StateView st, double rk)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n_fsr) return;
    const double *nf = g.xsnf + (size_t)g.fsr_mat[r] * g.G;
    double f = 0.0;
    for (int ig = 0; ig < g.G; ig++) f += rk * nf[ig] * st.phi[(size_t)ig * g.n_fsr + r];
    st.fs[r] = f;
}
void launch_fission_source(const GeomView &g, const StateView &st, double k, cudaStream_t s)
{
    { note_launch(); k_fission_source<<<(g.n_fsr + 255) / 256, 256, 0, s>>>(g, st, 1.0 / k); }
}

// sum_r sum_g phi V nuSigma_f   (transport_sweeper.cpp:104-117)
__global__ void k_total_fission(GeomView g, const double *phi, double *out)
{
    __shared__ double scratch[32];
    double acc = 0.0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < g.n_fsr; r += gridDim.x * blockDim.x) {
        const double *nf = g.xsnf + (size_t)g.fsr_mat[r] * g.G;
        double v = g.fsr_vol[r];
        for (int ig = 0; ig < g.G; ig++) acc += phi[(size_t)ig * g.n_fsr + r] * v * nf[ig];
    }
    acc = block_sum(acc, scratch);
    if (threadIdx.x == 0) atomicAdd(out, acc);
}
void launch_total_fission(const GeomView &g, const double *phi, double *out, cudaStream_t s)
{
    MOCGPU_CUDA(cudaMemsetAsync(out, 0, sizeof(double), s));
    { note_launch(); k_total_fission<<<grid_for(g.n_fsr, 256, 304), 256, 0, s>>>(g, phi, out); }
}

// Group source (source.cpp:41-112): src_r = chi_g fs_r + sum_{g'!=g} S(g<-g') phi_g'
// and the transport source with self-scatter (source_isotropic.cpp:21-57):
// qbar_r = (src_r + S(g<-g) phi_g,r) / (4 pi Sigma_tr,g). Also stages
// Sigma_t of this group per FSR for the sweep.
template <typename Real> __global__ void k_group_source(GeomView g, StateView st, int group)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n_fsr) return;
    const int G = g.G;
    const int m = g.fsr_mat[r];
    const double *srow = g.scat + ((size_t)m * G + group) * G;
    double src = g.xsch[(size_t)m * G + group] * st.fs[r];
    for (int gg = 0; gg < G; gg++)
        if (gg != group) src += srow[gg] * st.phi[(size_t)gg * g.n_fsr + r];
    st.src1g[r] = src;
    double xt = g.xstr[(size_t)m * G + group];
    double q = (src + st.phi[(size_t)group * g.n_fsr + r] * srow[group]) * (1.0 / (xt * kFpi));
    ((Real *)st.qbar)[r] = (Real)q;
    // the sweep's Sigma_t: XSMesh::expand with the split (xs_mesh.hpp:282-296);
    // the self-scatter source keeps the material's (source_isotropic.cpp:21-57)
    ((Real *)st.sigt)[r] = (Real)(st.split ? xt + st.split[r] : xt);
}

template <typename Real> __global__ void k_apply_tl(GeomView g, StateView st, int group, const double *tl)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n_fsr) return;
    const int G = g.G, m = g.fsr_mat[r];
    const double ph = st.phi[(size_t)group * g.n_fsr + r];
    double s = st.src1g[r] + tl[r];
    if (st.split) {
        double sp = 0.0;
        if (s < 0.0) {
            if (ph < 0.0) atomicOr(st.status, (unsigned)DEV_NEGATIVE_SPLIT_FLUX);
            sp = -s / ph;
            s = 0.0;
        }
        st.split[r] = sp;
    }
    st.src1g[r] = s;
    const double xt = g.xstr[(size_t)m * G + group];
    const double sgg = g.scat[((size_t)m * G + group) * G + group];
    ((Real *)st.qbar)[r] = (Real)((s + ph * sgg) * (1.0 / (xt * kFpi)));
    ((Real *)st.sigt)[r] = (Real)(st.split ? xt + st.split[r] : xt);
}
template <typename Real>
void launch_apply_transverse_leakage(const GeomView &g, const StateView &st, int group, const double *tl,
                                     cudaStream_t s)
{
    { note_launch(); k_apply_tl<Real><<<(g.n_fsr + 255) / 256, 256, 0, s>>>(g, st, group, tl); }
}
template void launch_apply_transverse_leakage<float>(const GeomView &, const StateView &, int, const double *,
                                                     cudaStream_t);
template void launch_apply_transverse_leakage<double>(const GeomView &, const StateView &, int, const double *,
                                                      cudaStream_t);
template <typename Real> void launch_group_source(const GeomView &g, const StateView &st, int group, cudaStream_t s)
{
    { note_launch(); k_group_source<Real><<<(g.n_fsr + 255) / 256, 256, 0, s>>>(g, st, group); }
}
template void launch_group_source<float>(const GeomView &, const StateView &, int, cudaStream_t);
template void launch_group_source<double>(const GeomView &, const StateView &, int, cudaStream_t);

// ---------------------------------------------------------------------------
// Attenuation 1 - exp(-tau).
// FP64: MOCC's linear-interpolated table on [-10, 0] with 10000 intervals and
// the library exponential outside it (exponential.hpp:56-112).
// FP32: a 4-term Taylor series of 1 - e^{-tau} for tau < 1/64 (relative error
// below 1e-9 there) and the fast hardware exponential above it.
struct ExpConst {
    double min, space, rspace;
};
__constant__ ExpConst c_exp;

__device__ __forceinline__ double attenuation(double tau, const double *tab)
{
    double v = -tau;
    if (v < c_exp.min || v > 0.0) return 1.0 - exp(v);
    int i = (int)((v - c_exp.min) * c_exp.rspace);
    if (i >= kExpN) i = kExpN - 1;
    v -= c_exp.space * i + c_exp.min;
    double d0 = __ldg(tab + i), d1 = __ldg(tab + i + 1);
    return 1.0 - (d0 + (d1 - d0) * v * c_exp.rspace);
}
__device__ __forceinline__ float attenuation(float tau, const double *)
{
    if (tau < 0.015625f) return tau * (1.0f - tau * (0.5f - tau * (0.16666667f - tau * 0.041666668f)));
    return 1.0f - __expf(-tau);
}

void set_exp_constants(double min, double space, double rspace)
{
    ExpConst c{min, space, rspace};
    MOCGPU_CUDA(cudaMemcpyToSymbol(c_exp, &c, sizeof(c)));
}

// ---------------------------------------------------------------------------
// One-group sweep of a range of tracks (moc_sweeper_kernel.inc.hpp:36-180):
// one thread per track, all polar angles of the track's azimuth in
// registers, forward then backward. The FSR tally of one segment is summed
// over the polar angles in registers before a single atomic add.
// Outgoing angular flux is written straight into the incoming slot of the
// reflected angle (Gauss-Seidel, boundary_condition.cpp:155-191) or into the
// outgoing buffer (Jacobi). With currents enabled the coarse-surface current
// and surface flux are tallied at the precomputed crossing events
// (moc_current_worker.hpp:202-264).
template <typename Real, int NPOL, bool GS, bool CUR>
__global__ void __launch_bounds__(128) k_sweep(GeomView g, StateView st, int group, int t0, int t1)
{
    int t = t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= t1) return;
    const Real *len = (const Real *)g.seg_len;
    const Real *sigt = (const Real *)st.sigt;
    const Real *qbar = (const Real *)st.qbar;
    Real *tally = (Real *)st.tally;
    Real *psi_in = (Real *)st.psi_in + (size_t)group * g.bc_per_group;
    Real *psi_out = (Real *)st.psi_out;
    const int set = g.trk_set[t];
    const int64_t b = g.seg_begin[t];
    const int n = (int)(g.seg_begin[t + 1] - b);
    const int bc0 = g.trk_bc0[t], bc1 = g.trk_bc1[t];
    const int ny_set = g.set_ny[set];

    Real rsin[NPOL], wt[NPOL], psi[NPOL];
    int af[NPOL], ab[NPOL];
    double cw[NPOL][2], fwt[NPOL][2];
#pragma unroll
    for (int p = 0; p < NPOL; p++) {
        const SetPolar sp = g.sp[set * NPOL + p];
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

    auto tally_events = [&](const int *pt, const int *code, int &ev, int ev_end, int k, double sign) {
        while (ev < ev_end && pt[ev] == k) {
            int c = code[ev];
            int surf = c >> 1, nrm = c & 1;
            double jc = 0.0, fc = 0.0;
#pragma unroll
            for (int p = 0; p < NPOL; p++) {
                jc += (double)psi[p] * cw[p][nrm];
                fc += (double)psi[p] * fwt[p][nrm];
            }
            atomicAdd(cur + surf, sign * jc);
            atomicAdd(sfl + surf, fc);
            ev++;
        }
    };
    auto store_out = [&](int ang, int idx, Real v) {
        if (GS) {
            // the reflected angle's entry, zeroed on a vacuum face
            // (BoundaryCondition::update, boundary_condition.cpp:155-191)
            const int face = idx < ny_set ? 0 : 1;
            const int tgt = g.wt_tgt[ang * 2 + face];
            psi_in[g.wt_tgt[3 * g.n_ang + ang * 2 + face] + idx] = tgt >= 0 ? v : (Real)0;
        } else {
            psi_out[g.bc_off[ang] + idx] = v;
        }
    };

    // forward
#pragma unroll
    for (int p = 0; p < NPOL; p++) psi[p] = psi_in[g.bc_off[af[p]] + bc0];
    int ev = 0, ev_end = 0;
    if (CUR) {
        ev = g.ev_fw_begin[t];
        ev_end = g.ev_fw_begin[t + 1];
        tally_events(g.ev_fw_pt, g.ev_fw_code, ev, ev_end, 0, 1.0);
    }
    for (int s = 0; s < n; s++) {
        const int r = g.seg_fsr[b + s];
        const Real tau0 = sigt[r] * len[b + s];
        const Real q = qbar[r];
        Real acc = 0;
#pragma unroll
        for (int p = 0; p < NPOL; p++) {
            Real e = attenuation(tau0 * rsin[p], g.exp_tab);
            Real d = (psi[p] - q) * e;
            psi[p] -= d;
            acc += d * wt[p];
        }
        atomicAdd(tally + r, acc);
        if (CUR) tally_events(g.ev_fw_pt, g.ev_fw_code, ev, ev_end, s + 1, 1.0);
    }
#pragma unroll
    for (int p = 0; p < NPOL; p++) store_out(af[p], bc1, psi[p]);

    // backward
#pragma unroll
    for (int p = 0; p < NPOL; p++) psi[p] = psi_in[g.bc_off[ab[p]] + bc1];
    if (CUR) {
        ev = g.ev_bw_begin[t];
        ev_end = g.ev_bw_begin[t + 1];
        tally_events(g.ev_bw_pt, g.ev_bw_code, ev, ev_end, n, -1.0);
    }
    for (int s = n - 1; s >= 0; s--) {
        const int r = g.seg_fsr[b + s];
        const Real tau0 = sigt[r] * len[b + s];
        const Real q = qbar[r];
        Real acc = 0;
#pragma unroll
        for (int p = 0; p < NPOL; p++) {
            Real e = attenuation(tau0 * rsin[p], g.exp_tab);
            Real d = (psi[p] - q) * e;
            psi[p] -= d;
            acc += d * wt[p];
        }
        atomicAdd(tally + r, acc);
        if (CUR) tally_events(g.ev_bw_pt, g.ev_bw_code, ev, ev_end, s, -1.0);
    }
#pragma unroll
    for (int p = 0; p < NPOL; p++) store_out(ab[p], bc0, psi[p]);
}

template <typename Real, int NPOL>
static void launch_sweep_np(const GeomView &g, const StateView &st, int group, int t0, int t1, bool gs, bool cur,
                            cudaStream_t s)
{
    int n = t1 - t0;
    if (n <= 0) return;
    int grid = (n + 127) / 128;
    if (gs) {
        if (cur) { note_launch(); k_sweep<Real, NPOL, true, true><<<grid, 128, 0, s>>>(g, st, group, t0, t1); }
        else { note_launch(); k_sweep<Real, NPOL, true, false><<<grid, 128, 0, s>>>(g, st, group, t0, t1); }
    } else {
        if (cur) { note_launch(); k_sweep<Real, NPOL, false, true><<<grid, 128, 0, s>>>(g, st, group, t0, t1); }
        else { note_launch(); k_sweep<Real, NPOL, false, false><<<grid, 128, 0, s>>>(g, st, group, t0, t1); }
    }
}

template <typename Real>
void launch_sweep(const GeomView &g, const StateView &st, int group, int t0, int t1, bool gs, bool cur,
                  cudaStream_t s)
{
    switch (g.pol) {
    case 1: launch_sweep_np<Real, 1>(g, st, group, t0, t1, gs, cur, s); break;
    case 2: launch_sweep_np<Real, 2>(g, st, group, t0, t1, gs, cur, s); break;
    case 3: launch_sweep_np<Real, 3>(g, st, group, t0, t1, gs, cur, s); break;
    case 4: launch_sweep_np<Real, 4>(g, st, group, t0, t1, gs, cur, s); break;
    default: throw Error(1, "unsupported number of polar angles per track set");
    }
}
template void launch_sweep<float>(const GeomView &, const StateView &, int, int, int, bool, bool, cudaStream_t);
template void launch_sweep<double>(const GeomView &, const StateView &, int, int, int, bool, bool, cudaStream_t);

// Jacobi boundary update: in(reflect(a, n)) <- out(a) on reflective faces,
// 0 on vacuum faces (boundary_condition.cpp:145-191).
template <typename Real> __global__ void k_jacobi_update(GeomView g, StateView st, int group)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.bc_per_group) return;
    // locate the angle owning entry i
    int lo = 0, hi = g.n_ang - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (g.bc_off[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    const int a = lo;
    const int idx = i - g.bc_off[a];
    Real *in = (Real *)st.psi_in + (size_t)group * g.bc_per_group;
    const Real *out = (const Real *)st.psi_out;
    const int face = (idx < g.wt_tgt[2 * g.n_ang + a]) ? 0 : 1;
    const int tgt = g.wt_tgt[a * 2 + face];
    const int base = g.wt_tgt[3 * g.n_ang + a * 2 + face];
    in[base + idx] = (tgt >= 0) ? out[i] : (Real)0;
}
template <typename Real> void launch_jacobi_update(const GeomView &g, const StateView &st, int group, cudaStream_t s)
{
    { note_launch(); k_jacobi_update<Real><<<(g.bc_per_group + 255) / 256, 256, 0, s>>>(g, st, group); }
}
template void launch_jacobi_update<float>(const GeomView &, const StateView &, int, cudaStream_t);
template void launch_jacobi_update<double>(const GeomView &, const StateView &, int, cudaStream_t);

// phi = tally / (Sigma_t V) + 4 pi qbar (moc_sweeper_kernel.inc.hpp:165-173),
// then the self-scatter update of qbar for the next inner iteration.
template <typename Real> __global__ void k_sweep_epilogue(GeomView g, StateView st, int group, int update_q)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n_fsr) return;
    Real *tally = (Real *)st.tally;
    Real *qbar = (Real *)st.qbar;
    const Real *sigt = (const Real *)st.sigt;
    double q = (double)qbar[r];
    double ph = (double)tally[r] / ((double)sigt[r] * g.fsr_vol[r]) + q * kFpi;
    st.phi[(size_t)group * g.n_fsr + r] = ph;
    tally[r] = (Real)0;
    if (update_q) {
        const int G = g.G, m = g.fsr_mat[r];
        double sgg = g.scat[((size_t)m * G + group) * G + group];
        double xt = g.xstr[(size_t)m * G + group];
        qbar[r] = (Real)((st.src1g[r] + ph * sgg) * (1.0 / (xt * kFpi)));
    }
}
template <typename Real>
void launch_sweep_epilogue(const GeomView &g, const StateView &st, int group, bool update_q, cudaStream_t s)
{
    { note_launch(); k_sweep_epilogue<Real><<<(g.n_fsr + 255) / 256, 256, 0, s>>>(g, st, group, update_q ? 1 : 0); }
}
template void launch_sweep_epilogue<float>(const GeomView &, const StateView &, int, bool, cudaStream_t);
template void launch_sweep_epilogue<double>(const GeomView &, const StateView &, int, bool, cudaStream_t);

void launch_zero_radial_currents(const GeomView &g, const StateView &st, int group, cudaStream_t s)
{
    MOCGPU_CUDA(cudaMemsetAsync(st.cur + (size_t)group * g.n_surf, 0, sizeof(double) * g.n_surf, s));
    MOCGPU_CUDA(cudaMemsetAsync(st.sflux + (size_t)group * g.n_surf, 0, sizeof(double) * g.n_surf, s));
    MOCGPU_CUDA(cudaMemsetAsync(st.cur32, 0, sizeof(float) * 2 * kCurCopies * g.n_surf, s));
}

// Currents per unit area on the x/y-normal surfaces (moc_current_worker.hpp:272-318),
// with the FP32 sweep's tallies folded in (and cleared for the next group).
__device__ __forceinline__ void normalize_surface(const GeomView &g, const StateView &st, int group, int i,
                                                  const double *area)
{
    const size_t k = (size_t)group * g.n_surf + i;
    float c = 0.f, f = 0.f;
#pragma unroll
    for (int j = 0; j < kCurCopies; j++) {
        c += st.cur32[(size_t)j * g.n_surf + i];
        f += st.sfl32[(size_t)j * g.n_surf + i];
        st.cur32[(size_t)j * g.n_surf + i] = 0.f;
        st.sfl32[(size_t)j * g.n_surf + i] = 0.f;
    }
    st.cur[k] = (st.cur[k] + (double)c) / area[i];
    st.sflux[k] = (st.sflux[k] + (double)f) / area[i];
}
__global__ void k_normalize_currents(GeomView g, StateView st, int group, const double *area)
{
    int i = g.nx * g.ny + blockIdx.x * blockDim.x + threadIdx.x;
    int end = (g.nx + 1) * g.ny + (g.ny + 1) * g.nx + g.nx * g.ny;
    if (i >= end) return;
    normalize_surface(g, st, group, i, area);
}
void launch_normalize_currents(const GeomView &g, const StateView &st, int group, const double *area, cudaStream_t s)
{
    int n = (g.nx + 1) * g.ny + (g.ny + 1) * g.nx;
    { note_launch(); k_normalize_currents<<<(n + 255) / 256, 256, 0, s>>>(g, st, group, area); }
}

// ---------------------------------------------------------------------------
// Volume-averaged pin flux per group (moc_sweeper.cpp:293-326).
__global__ void k_pin_flux(GeomView g, const double *phi, double *cflux)
{
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.n_pin * g.G) return;
    int ig = idx / g.n_pin, ip = idx % g.n_pin;
    double v = 0.0, pf = 0.0;
    for (int r = g.pin_first_reg[ip]; r < g.pin_first_reg[ip + 1]; r++) {
        v += g.fsr_vol[r];
        pf += phi[(size_t)ig * g.n_fsr + r] * g.fsr_vol[r];
    }
    cflux[(size_t)ig * g.n_pin + g.pin_cell[ip]] = pf / v;
}
void launch_pin_flux(const GeomView &g, const double *phi, double *cflux, cudaStream_t s)
{
    int n = g.n_pin * g.G;
    { note_launch(); k_pin_flux<<<(n + 255) / 256, 256, 0, s>>>(g, phi, cflux); }
}

// Rescale FSR fluxes by the coarse/fine pin-flux ratio (moc_sweeper.cpp:360-433).
// A non-positive coarse flux raises a status flag and leaves that pin alone.
__global__ void k_set_pin_flux(GeomView g, double *phi, const double *cflux, double *resid, unsigned *status)
{
    __shared__ double scratch[32];
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    double e2 = 0.0;
    if (idx < g.n_pin * g.G) {
        int ig = idx / g.n_pin, ip = idx % g.n_pin;
        double c = cflux[(size_t)ig * g.n_pin + g.pin_cell[ip]];
        if (!(c > 0.0)) {
            atomicOr(status, (unsigned)DEV_NONPOSITIVE_PIN_FLUX);
        } else {
            double fm = 0.0;
            int r0 = g.pin_first_reg[ip], r1 = g.pin_first_reg[ip + 1];
            for (int r = r0; r < r1; r++) fm += phi[(size_t)ig * g.n_fsr + r] * g.fsr_area[r];
            fm /= g.pin_area[ip];
            double e = c - fm, f = c / fm;
            for (int r = r0; r < r1; r++) phi[(size_t)ig * g.n_fsr + r] *= f;
            e2 = e * e;
        }
    }
    e2 = block_sum(e2, scratch);
    if (threadIdx.x == 0 && resid) atomicAdd(resid, e2);
}
void launch_set_pin_flux(const GeomView &g, double *phi, const double *cflux, double *resid, unsigned *status,
                         cudaStream_t s)
{
    int n = g.n_pin * g.G;
    { note_launch(); k_set_pin_flux<<<(n + 255) / 256, 256, 0, s>>>(g, phi, cflux, resid, status); }
}

// Flux-weighted pin homogenisation (xs_mesh_homogenized.cpp:261-363).
__device__ void homogenize_pin(const GeomView &g, const double *phi, const CmfdView &c, int idx)
{
    // one (pin, group) pair per thread: the group's flux-weighted XS, its
    // fission-source-weighted chi and its scattering row
    const double *fsr_area = g.fsr_area;
    const int G = g.G;
    if (idx >= g.n_pin * G) return;
    const int ip = idx / G, ig = idx % G;
    const int cell = g.pin_cell[ip];
    const int r0 = g.pin_first_reg[ip], r1 = g.pin_first_reg[ip + 1];
    double fs_sum = 0.0;
    for (int r = r0; r < r1; r++) {
        const double *nf = g.xsnf + (size_t)g.fsr_mat[r] * G;
        double f = 0.0;
        for (int gg = 0; gg < G; gg++) f += nf[gg] * phi[(size_t)gg * g.n_fsr + r] * fsr_area[r];
        fs_sum += f;
    }
    double fvs = 0.0, xt = 0.0, xnf = 0.0, xf = 0.0, xch = 0.0;
    for (int r = r0; r < r1; r++) {
        int m = g.fsr_mat[r];
        double v = fsr_area[r], fl = phi[(size_t)ig * g.n_fsr + r];
        fvs += v * fl;
        xt += v * fl * g.xstr[(size_t)m * G + ig];
        xnf += v * fl * g.xsnf[(size_t)m * G + ig];
        xf += v * fl * g.xsf[(size_t)m * G + ig];
        double fsr_fs = 0.0;
        for (int gg = 0; gg < G; gg++) fsr_fs += g.xsnf[(size_t)m * G + gg] * phi[(size_t)gg * g.n_fsr + r] * v;
        xch += fsr_fs * g.xsch[(size_t)m * G + ig];
    }
    double self = 0.0;
    for (int gg = 0; gg < G; gg++) {
        double num = 0.0, den = 0.0;
        for (int r = r0; r < r1; r++) {
            int m = g.fsr_mat[r];
            double v = fsr_area[r], fl = phi[(size_t)gg * g.n_fsr + r];
            den += fl * v;
            num += g.scat[((size_t)m * G + ig) * G + gg] * v * fl;
        }
        if (num > 0.0) num /= den;
        c.scat[((size_t)cell * G + ig) * G + gg] = num;
        if (gg == ig) self = num;
    }
    const double xs_tr = xt / fvs;
    c.xstr[(size_t)cell * G + ig] = xs_tr;
    c.xsnf[(size_t)cell * G + ig] = xnf / fvs;
    c.xsf[(size_t)cell * G + ig] = xf / fvs;
    c.xsch[(size_t)cell * G + ig] = (fs_sum > 0.0) ? xch / fs_sum : xch;
    c.xsrm[(size_t)cell * G + ig] = xs_tr - self;
}
__global__ void k_homogenize(GeomView g, const double *phi, CmfdView c)
{
    homogenize_pin(g, phi, c, blockIdx.x * blockDim.x + threadIdx.x);
}
void launch_homogenize(const GeomView &g, const double *phi, const CmfdView &c, cudaStream_t s)
{
    { note_launch(); k_homogenize<<<(g.n_pin * g.G + 127) / 128, 128, 0, s>>>(g, phi, c); }
}

// ---------------------------------------------------------------------------
// Fission-source change after MOCC's Normalize() of both vectors
// (eigen_solver.cpp:171-184, util/utils.hpp:29-51). red[0..3] receive
// (count>0, sum) of fs and fs_prev; red[4] the squared difference.
__global__ void k_psi_err_sums(GeomView g, const double *fs, const double *fp, double *red)
{
    __shared__ double scratch[64];
    double na = 0, sa = 0, nb = 0, sb = 0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < g.n_fsr; r += gridDim.x * blockDim.x) {
        double a = fs[r], b = fp[r];
        if (a > 0.0) na += 1.0;
        sa += a;
        if (b > 0.0) nb += 1.0;
        sb += b;
    }
    block_sum2(na, sa, scratch);
    block_sum2(nb, sb, scratch);
    if (threadIdx.x == 0) {
        atomicAdd(red + 0, na);
        atomicAdd(red + 1, sa);
        atomicAdd(red + 2, nb);
        atomicAdd(red + 3, sb);
    }
}
__global__ void k_psi_err_diff(GeomView g, const double *fs, const double *fp, double *red)
{
    __shared__ double scratch[32];
    double fa = red[0] / red[1], fb = red[2] / red[3];
    double acc = 0.0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < g.n_fsr; r += gridDim.x * blockDim.x) {
        double e = fs[r] * fa - fp[r] * fb;
        acc += e * e;
    }
    acc = block_sum(acc, scratch);
    if (threadIdx.x == 0) atomicAdd(red + 4, acc);
}
void launch_psi_error(const GeomView &g, const double *fs, const double *fs_prev, double *red, cudaStream_t s)
{
    MOCGPU_CUDA(cudaMemsetAsync(red, 0, 5 * sizeof(double), s));
    int grid = grid_for(g.n_fsr, 256, 304);
    { note_launch(); k_psi_err_sums<<<grid, 256, 0, s>>>(g, fs, fs_prev, red); }
    { note_launch(); k_psi_err_diff<<<grid, 256, 0, s>>>(g, fs, fs_prev, red); }
}

// sqrt(sum (phi - phi_old)^2)  (transport_sweeper.cpp:210-223); out = sum only
__global__ void k_flux_residual(GeomView g, const double *a, const double *b, double *out)
{
    __shared__ double scratch[32];
    double acc = 0.0;
    int64_t n = (int64_t)g.n_fsr * g.G;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double e = a[i] - b[i];
        acc += e * e;
    }
    acc = block_sum(acc, scratch);
    if (threadIdx.x == 0) atomicAdd(out, acc);
}
void launch_flux_residual(const GeomView &g, const StateView &st, double *out, cudaStream_t s)
{
    MOCGPU_CUDA(cudaMemsetAsync(out, 0, sizeof(double), s));
    { note_launch(); k_flux_residual<<<grid_for((int64_t)g.n_fsr * g.G, 256, 304), 256, 0, s>>>(g, st.phi, st.phi_old, out); }
}

// Fission-rate pin powers (transport_sweeper.cpp:140-193): pow[cell] gets
// sum phi Sigma_f V over the pin's FSRs; pow[n_pin] gets the total.
__global__ void k_pin_power(GeomView g, const double *phi, double *pow)
{
    __shared__ double scratch[32];
    int ip = blockIdx.x * blockDim.x + threadIdx.x;
    double tot = 0.0;
    if (ip < g.n_pin) {
        double p = 0.0;
        for (int r = g.pin_first_reg[ip]; r < g.pin_first_reg[ip + 1]; r++) {
            const double *xf = g.xsf + (size_t)g.fsr_mat[r] * g.G;
            double fp = 0.0;
            for (int ig = 0; ig < g.G; ig++) fp += phi[(size_t)ig * g.n_fsr + r] * xf[ig] * g.fsr_vol[r];
            p += fp;
        }
        pow[g.pin_cell[ip]] = p;
        tot = p;
    }
    tot = block_sum(tot, scratch);
    if (threadIdx.x == 0) atomicAdd(pow + g.n_pin, tot);
}
void launch_pin_power(const GeomView &g, const double *phi, double *pow, cudaStream_t s)
{
    MOCGPU_CUDA(cudaMemsetAsync(pow + g.n_pin, 0, sizeof(double), s));
    { note_launch(); k_pin_power<<<(g.n_pin + 255) / 256, 256, 0, s>>>(g, phi, pow); }
}

// ===========================================================================
// Batched forms: the same arithmetic for every active solve of a batch, one
// solve per blockIdx.y; per-solve scalars (k, total fission, error sums) live
// in each solve's StateView::red so nothing returns to the host between
// launches. Solves with fewer groups than the group being processed skip it.
#define BATCH_SLOT                                                                                                   \
    if ((int)blockIdx.y >= *b.n_act) return;                                                                         \
    const int slot = b.act[blockIdx.y];                                                                              \
    const GeomView &g = b.gv[slot];                                                                                  \
    const StateView &st = b.sv[slot];                                                                                \
    if (st.red[RED_DONE] != 0.0) return; /* finished: frozen */

static dim3 bgrid(int n, int block, int cap) { return dim3((unsigned)((n + block - 1) / block), (unsigned)cap); }

__global__ void kb_fission_source(BatchViews b)
{
    BATCH_SLOT
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n_fsr) return;
    const double rk = 1.0 / st.red[RED_K];
    const double *nf = g.xsnf + (size_t)g.fsr_mat[r] * g.G;
    double f = 0.0;
    for (int ig = 0; ig < g.G; ig++) f += rk * nf[ig] * st.phi[(size_t)ig * g.n_fsr + r];
    st.fs[r] = f;
}
void launch_b_fission_source(const BatchViews &b, cudaStream_t s)
{
    note_launch();
    kb_fission_source<<<bgrid(b.max_fsr, 256, b.cap), 256, 0, s>>>(b);
}

__global__ void kb_copy_old(BatchViews b)
{
    BATCH_SLOT
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n_fsr) return;
    st.fs_prev[r] = st.fs[r];
    for (int ig = 0; ig < g.G; ig++) st.phi_old[(size_t)ig * g.n_fsr + r] = st.phi[(size_t)ig * g.n_fsr + r];
}
void launch_b_copy_old(const BatchViews &b, cudaStream_t s)
{
    note_launch();
    kb_copy_old<<<bgrid(b.max_fsr, 256, b.cap), 256, 0, s>>>(b);
}

template <typename Real> __global__ void kb_group_source(BatchViews b, int group)
{
    BATCH_SLOT
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n_fsr || group >= g.G) return;
    const int G = g.G;
    const int m = g.fsr_mat[r];
    const double *srow = g.scat + ((size_t)m * G + group) * G;
    double src = g.xsch[(size_t)m * G + group] * st.fs[r];
    for (int gg = 0; gg < G; gg++)
        if (gg != group) src += srow[gg] * st.phi[(size_t)gg * g.n_fsr + r];
    st.src1g[r] = src;
    double xt = g.xstr[(size_t)m * G + group];
    double q = (src + st.phi[(size_t)group * g.n_fsr + r] * srow[group]) * (1.0 / (xt * kFpi));
    ((Real *)st.qbar)[r] = (Real)q;
    ((Real *)st.sigt)[r] = (Real)xt;
}
template <typename Real> void launch_b_group_source(const BatchViews &b, int group, cudaStream_t s)
{
    note_launch();
    kb_group_source<Real><<<bgrid(b.max_fsr, 256, b.cap), 256, 0, s>>>(b, group);
}
template void launch_b_group_source<float>(const BatchViews &, int, cudaStream_t);
template void launch_b_group_source<double>(const BatchViews &, int, cudaStream_t);

template <typename Real> __global__ void kb_epilogue(BatchViews b, int group, int update_q)
{
    BATCH_SLOT
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= g.n_fsr || group >= g.G) return;
    Real *tally = (Real *)st.tally;
    Real *qbar = (Real *)st.qbar;
    const Real *sigt = (const Real *)st.sigt;
    double q = (double)qbar[r];
    double ph = (double)tally[r] / ((double)sigt[r] * g.fsr_vol[r]) + q * kFpi;
    st.phi[(size_t)group * g.n_fsr + r] = ph;
    tally[r] = (Real)0;
    if (update_q) {
        const int G = g.G, m = g.fsr_mat[r];
        double sgg = g.scat[((size_t)m * G + group) * G + group];
        double xt = g.xstr[(size_t)m * G + group];
        qbar[r] = (Real)((st.src1g[r] + ph * sgg) * (1.0 / (xt * kFpi)));
    }
}
template <typename Real> void launch_b_epilogue(const BatchViews &b, int group, bool update_q, cudaStream_t s)
{
    note_launch();
    kb_epilogue<Real><<<bgrid(b.max_fsr, 256, b.cap), 256, 0, s>>>(b, group, update_q ? 1 : 0);
}
template void launch_b_epilogue<float>(const BatchViews &, int, bool, cudaStream_t);
template void launch_b_epilogue<double>(const BatchViews &, int, bool, cudaStream_t);

__global__ void kb_zero_currents(BatchViews b, int group)
{
    BATCH_SLOT
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n_surf || group >= g.G) return;
    st.cur[(size_t)group * g.n_surf + i] = 0.0;
    st.sflux[(size_t)group * g.n_surf + i] = 0.0;
    for (int j = 0; j < kCurCopies; j++) {
        st.cur32[(size_t)j * g.n_surf + i] = 0.f;
        st.sfl32[(size_t)j * g.n_surf + i] = 0.f;
    }
}
void launch_b_zero_currents(const BatchViews &b, int group, cudaStream_t s)
{
    note_launch();
    kb_zero_currents<<<bgrid(b.max_surf, 256, b.cap), 256, 0, s>>>(b, group);
}

// Radial surfaces only: the axial ones are never tallied in 2-D
// (moc_sweeper.cpp:206-221 normalises every surface; axial entries stay 0).
__global__ void kb_normalize_currents(BatchViews b, int group)
{
    BATCH_SLOT
    if (group >= g.G) return;
    const double *area = b.surf_area[slot];
    int i = g.nx * g.ny + blockIdx.x * blockDim.x + threadIdx.x;
    int end = (g.nx + 1) * g.ny + (g.ny + 1) * g.nx + g.nx * g.ny;
    if (blockIdx.x == 0 && threadIdx.x == 0) st.red[RED_HAS_RADIAL] = 1.0;
    if (i >= end) return;
    normalize_surface(g, st, group, i, area);
}
void launch_b_normalize_currents(const BatchViews &b, int group, cudaStream_t s)
{
    note_launch();
    kb_normalize_currents<<<bgrid(b.max_surf, 256, b.cap), 256, 0, s>>>(b, group);
}

__global__ void kb_pin_flux(BatchViews b)
{
    BATCH_SLOT
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.n_pin * g.G) return;
    int ig = idx / g.n_pin, ip = idx % g.n_pin;
    double v = 0.0, pf = 0.0;
    for (int r = g.pin_first_reg[ip]; r < g.pin_first_reg[ip + 1]; r++) {
        v += g.fsr_vol[r];
        pf += st.phi[(size_t)ig * g.n_fsr + r] * g.fsr_vol[r];
    }
    st.cflux[(size_t)ig * g.n_pin + g.pin_cell[ip]] = pf / v;
}
void launch_b_pin_flux(const BatchViews &b, cudaStream_t s)
{
    note_launch();
    kb_pin_flux<<<bgrid(b.max_pin * b.max_g, 256, b.cap), 256, 0, s>>>(b);
}

__global__ void kb_homogenize(BatchViews b)
{
    BATCH_SLOT
    homogenize_pin(g, st.phi, b.cv[slot], blockIdx.x * blockDim.x + threadIdx.x);
}
void launch_b_homogenize(const BatchViews &b, cudaStream_t s)
{
    note_launch();
    kb_homogenize<<<bgrid(b.max_pin * b.max_g, 64, b.cap), 64, 0, s>>>(b);
}

__global__ void kb_set_pin_flux(BatchViews b)
{
    BATCH_SLOT
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= g.n_pin * g.G) return;
    int ig = idx / g.n_pin, ip = idx % g.n_pin;
    double c = st.cflux[(size_t)ig * g.n_pin + g.pin_cell[ip]];
    if (!(c > 0.0)) {
        atomicOr(st.status, (unsigned)DEV_NONPOSITIVE_PIN_FLUX);
        return;
    }
    double fm = 0.0;
    int r0 = g.pin_first_reg[ip], r1 = g.pin_first_reg[ip + 1];
    for (int r = r0; r < r1; r++) fm += st.phi[(size_t)ig * g.n_fsr + r] * g.fsr_area[r];
    fm /= g.pin_area[ip];
    double f = c / fm;
    for (int r = r0; r < r1; r++) st.phi[(size_t)ig * g.n_fsr + r] *= f;
}
void launch_b_set_pin_flux(const BatchViews &b, cudaStream_t s)
{
    note_launch();
    kb_set_pin_flux<<<bgrid(b.max_pin * b.max_g, 256, b.cap), 256, 0, s>>>(b);
}

// Per solve: total fission of the new and the old flux
// (transport_sweeper.cpp:104-117), k <- k * new / old, then the fission
// source at the new k (eigen_solver.cpp:242-250). One CTA per solve.
__global__ void kb_k_update(BatchViews b)
{
    __shared__ double scratch[64];
    if ((int)blockIdx.x >= *b.n_act) return;
    const int slot = b.act[blockIdx.x];
    const GeomView &g = b.gv[slot];
    const StateView &st = b.sv[slot];
    if (st.red[RED_DONE] != 0.0) return; // finished: frozen
    const int G = g.G;
    double tn = 0.0, to = 0.0;
    for (int r = threadIdx.x; r < g.n_fsr; r += blockDim.x) {
        const double *nf = g.xsnf + (size_t)g.fsr_mat[r] * G;
        double v = g.fsr_vol[r];
        for (int ig = 0; ig < G; ig++) {
            tn += st.phi[(size_t)ig * g.n_fsr + r] * v * nf[ig];
            to += st.phi_old[(size_t)ig * g.n_fsr + r] * v * nf[ig];
        }
    }
    block_sum2(tn, to, scratch);
    const double k = st.red[RED_K];
    const double knew = k * tn / to;
    __syncthreads();
    if (threadIdx.x == 0) {
        st.red[RED_TF_NEW] = tn;
        st.red[RED_TF_OLD] = to;
        st.red[RED_K_PREV] = k;
        st.red[RED_K] = knew;
    }
    const double rk = 1.0 / knew;
    for (int r = threadIdx.x; r < g.n_fsr; r += blockDim.x) {
        const double *nf = g.xsnf + (size_t)g.fsr_mat[r] * G;
        double f = 0.0;
        for (int ig = 0; ig < G; ig++) f += rk * nf[ig] * st.phi[(size_t)ig * g.n_fsr + r];
        st.fs[r] = f;
    }
}
void launch_b_k_update(const BatchViews &b, cudaStream_t s)
{
    note_launch();
    kb_k_update<<<b.cap, 256, 0, s>>>(b);
}

// Per solve: |k - k_prev| and the fission-source change after MOCC's
// Normalize() of both sources (eigen_solver.cpp:171-184). One CTA per solve.
__global__ void kb_errors(BatchViews b)
{
    __shared__ double scratch[64];
    if ((int)blockIdx.x >= *b.n_act) return;
    const int slot = b.act[blockIdx.x];
    const GeomView &g = b.gv[slot];
    const StateView &st = b.sv[slot];
    if (st.red[RED_DONE] != 0.0) return; // finished: frozen
    double na = 0, sa = 0, nb = 0, sb = 0;
    for (int r = threadIdx.x; r < g.n_fsr; r += blockDim.x) {
        double a = st.fs[r], c = st.fs_prev[r];
        if (a > 0.0) na += 1.0;
        sa += a;
        if (c > 0.0) nb += 1.0;
        sb += c;
    }
    block_sum2(na, sa, scratch);
    block_sum2(nb, sb, scratch);
    const double fa = na / sa, fb = nb / sb;
    double acc = 0.0, dummy = 0.0;
    for (int r = threadIdx.x; r < g.n_fsr; r += blockDim.x) {
        double e = st.fs[r] * fa - st.fs_prev[r] * fb;
        acc += e * e;
    }
    block_sum2(acc, dummy, scratch);
    if (threadIdx.x == 0) {
        st.red[RED_ERR_K] = fabs(st.red[RED_K] - st.red[RED_K_PREV]);
        st.red[RED_ERR_PSI] = sqrt(acc / st.red[RED_N_FISSILE]);
        if (!isfinite(st.red[RED_K])) atomicOr(st.status, (unsigned)DEV_NAN);
    }
}
void launch_b_errors(const BatchViews &b, cudaStream_t s)
{
    note_launch();
    kb_errors<<<b.cap, 256, 0, s>>>(b);
}

__global__ void kb_retire(BatchViews b, double *out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *b.n_act) return;
    const int slot = b.act[i];
    const StateView &st = b.sv[slot];
    double *red = st.red;
    if (red[RED_DONE] != 0.0) return; // ended in an earlier replay: its row stays as it was
    const double it = red[RED_ITERS] + 1.0;
    red[RED_ITERS] = it;
    const double k = red[RED_K], ek = red[RED_ERR_K], ep = red[RED_ERR_PSI];
    const unsigned status = *st.status;
    int code = DONE_RUNNING;
    if (status & DEV_NONPOSITIVE_PIN_FLUX) code = DONE_NONPOSITIVE;
    else if ((status & DEV_NAN) || !isfinite(k)) code = DONE_NAN;
    else if (ek < red[RED_K_TOL] && ep < red[RED_PSI_TOL] && it - 1.0 >= red[RED_MIN_ITER]) code = DONE_CONVERGED;
    else if (it >= red[RED_MAX_ITER]) code = DONE_MAX_ITER;
    red[RED_DONE] = (double)code;
    double *o = out + (size_t)slot * kSummaryStride;
    o[0] = k;
    o[1] = ek;
    o[2] = ep;
    o[3] = (double)status;
    o[4] = red[RED_CMFD_ITS];
    o[5] = red[RED_HAS_RADIAL];
    o[6] = (double)code;
    o[7] = it;
}
void launch_b_retire(const BatchViews &b, double *out, cudaStream_t s)
{
    note_launch();
    kb_retire<<<(b.cap + 127) / 128, 128, 0, s>>>(b, out);
}

// Fission-rate pin powers of every active solve (transport_sweeper.cpp:140-193):
// row `slot` of out gets sum phi Sigma_f V per coarse cell and, in entry
// n_pin, their total. One CTA per solve.
__global__ void kb_pin_powers(BatchViews b, double *out, int stride)
{
    __shared__ double scratch[32];
    if ((int)blockIdx.x >= *b.n_act) return;
    const int slot = b.act[blockIdx.x];
    const GeomView &g = b.gv[slot];
    const StateView &st = b.sv[slot];
    if (st.red[RED_DONE] != 0.0) return; // finished: frozen
    double *row = out + (size_t)slot * stride;
    double tot = 0.0;
    for (int ip = threadIdx.x; ip < g.n_pin; ip += blockDim.x) {
        double p = 0.0;
        for (int r = g.pin_first_reg[ip]; r < g.pin_first_reg[ip + 1]; r++) {
            const double *xf = g.xsf + (size_t)g.fsr_mat[r] * g.G;
            double fp = 0.0;
            for (int ig = 0; ig < g.G; ig++) fp += st.phi[(size_t)ig * g.n_fsr + r] * xf[ig] * g.fsr_vol[r];
            p += fp;
        }
        row[g.pin_cell[ip]] = p;
        tot += p;
    }
    tot = block_sum(tot, scratch);
    if (threadIdx.x == 0) row[g.n_pin] = tot;
}
void launch_b_pin_powers(const BatchViews &b, double *out, int stride, cudaStream_t s)
{
    note_launch();
    kb_pin_powers<<<b.cap, 128, 0, s>>>(b, out, stride);
}

} // namespace mocgpu
