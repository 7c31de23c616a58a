// Bundled work-unit MoC sweep: single-solve launchers and the batched
// launcher's dispatch over streaming shapes (the kernels are in
// sweep_fast.cuh).
#include "sweep_fast.cuh"

namespace mocgpu {

template <typename Real> size_t fast_sweep_smem(const FastView &fv)
{
    int nwarps = 2 * fv.bundles_per_unit;
    return (size_t)nwarps * ring_bytes<Real, DefaultShape>() + (size_t)fv.max_local * fsr_slot_bytes<Real>();
}
template size_t fast_sweep_smem<float>(const FastView &);
template size_t fast_sweep_smem<double>(const FastView &);

template <typename Real, int NPOL, bool GS, int CUR>
static void launch_one(const GeomView &g, const FastView &fv, const StateView &st, int group, int wu0, int wu1,
                       cudaStream_t s)
{
    auto k = k_sweep_fast<Real, NPOL, GS, CUR>;
    size_t smem = fast_sweep_smem<Real>(fv);
    ensure_smem_limit((const void *)k, smem);
    int threads = 64 * fv.bundles_per_unit;
    k<<<wu1 - wu0, threads, smem, s>>>(g, fv, st, group, wu0);
}

template <typename Real, int NPOL>
static void launch_np(const GeomView &g, const FastView &fv, const StateView &st, int group, int wu0, int wu1, bool gs,
                      int cur, cudaStream_t s)
{
    if (gs && !cur) launch_one<Real, NPOL, true, 0>(g, fv, st, group, wu0, wu1, s);
    else if (gs && cur == 2) launch_one<Real, NPOL, true, 2>(g, fv, st, group, wu0, wu1, s);
    else if (gs && cur) launch_one<Real, NPOL, true, 1>(g, fv, st, group, wu0, wu1, s);
    else if (!gs && !cur) launch_one<Real, NPOL, false, 0>(g, fv, st, group, wu0, wu1, s);
    else launch_one<Real, NPOL, false, 1>(g, fv, st, group, wu0, wu1, s);
}

template <typename Real>
void launch_sweep_fast(const GeomView &g, const FastView &fv, const StateView &st, int group, int wu0, int wu1,
                       bool gs, int cur, cudaStream_t s)
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
template void launch_sweep_fast<float>(const GeomView &, const FastView &, const StateView &, int, int, int, bool, int,
                                       cudaStream_t);
template void launch_sweep_fast<double>(const GeomView &, const FastView &, const StateView &, int, int, int, bool,
                                        int, cudaStream_t);

} // namespace mocgpu

namespace mocgpu {

void sweep_shape_info(int shape, int *rows, int *stages)
{
    if (shape < 0 || shape >= kSweepShapeCount) throw Error(1, "no batched sweep shape " + std::to_string(shape));
    *rows = kShapeRows[shape];
    *stages = kShapeStages[shape];
}

template <typename Real> void prepare_b_sweep(int pol, int bundles_per_unit, int max_local, int shape)
{
    if (shape == 0) return prepare_batched_shape<Real, ShapeN<0>>(pol, bundles_per_unit, max_local);
    if (sizeof(Real) != 4) throw Error(1, "the FP64 batched sweep is built in shape 0 only");
    if (!prepare_b_sweep_shapes_a(shape, pol, bundles_per_unit, max_local) &&
        !prepare_b_sweep_shapes_b(shape, pol, bundles_per_unit, max_local))
        throw Error(1, "no batched sweep shape " + std::to_string(shape));
}
template void prepare_b_sweep<float>(int, int, int, int);
template void prepare_b_sweep<double>(int, int, int, int);

template <typename Real>
void launch_b_sweep(const BatchViews &b, const int2 *items, const int *n_items, int max_items, int group, int cur,
                    int pol, int bundles_per_unit, int max_local, int shape, int *counter, cudaStream_t s)
{
    if (max_items <= 0) return;
    note_launch_external();
    if (shape == 0)
        return launch_batched_shape<Real, ShapeN<0>>(b, items, n_items, max_items, group, cur, pol, bundles_per_unit,
                                                     max_local, counter, s);
    if (sizeof(Real) != 4) throw Error(1, "the FP64 batched sweep is built in shape 0 only");
    if (!launch_b_sweep_shapes_a(shape, b, items, n_items, max_items, group, cur, pol, bundles_per_unit, max_local,
                                 counter, s) &&
        !launch_b_sweep_shapes_b(shape, b, items, n_items, max_items, group, cur, pol, bundles_per_unit, max_local,
                                 counter, s))
        throw Error(1, "no batched sweep shape " + std::to_string(shape));
}
template void launch_b_sweep<float>(const BatchViews &, const int2 *, const int *, int, int, int, int, int, int, int,
                                    int *, cudaStream_t);
template void launch_b_sweep<double>(const BatchViews &, const int2 *, const int *, int, int, int, int, int, int, int,
                                     int *, cudaStream_t);

} // namespace mocgpu
