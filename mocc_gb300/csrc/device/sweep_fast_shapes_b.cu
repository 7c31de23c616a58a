// FP32 batched sweep in streaming shapes 3 and 4 (a translation unit of its
// own so that the kernel instances compile in parallel with the others).
#include "sweep_fast.cuh"

namespace mocgpu {

bool prepare_b_sweep_shapes_b(int shape, int pol, int bundles_per_unit, int max_local)
{
    switch (shape) {
    case 3: prepare_batched_shape<float, ShapeN<3>>(pol, bundles_per_unit, max_local); return true;
    case 4: prepare_batched_shape<float, ShapeN<4>>(pol, bundles_per_unit, max_local); return true;
    default: return false;
    }
}

bool launch_b_sweep_shapes_b(int shape, const BatchViews &b, const int2 *items, const int *n_items, int max_items,
                              int group, int cur, int pol, int bundles_per_unit, int max_local, int *counter,
                              cudaStream_t s)
{
    switch (shape) {
    case 3:
        launch_batched_shape<float, ShapeN<3>>(b, items, n_items, max_items, group, cur, pol, bundles_per_unit,
                                               max_local, counter, s);
        return true;
    case 4:
        launch_batched_shape<float, ShapeN<4>>(b, items, n_items, max_items, group, cur, pol, bundles_per_unit,
                                               max_local, counter, s);
        return true;
    default: return false;
    }
}

} // namespace mocgpu
