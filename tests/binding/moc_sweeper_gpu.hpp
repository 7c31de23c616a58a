// The binding a MOCC build would add next to MoCSweeper: a TransportSweeper
// (src/core/transport_sweeper.hpp:41-351) whose every duty forwards to the
// C ABI of include/mocgpu.h. Compiled and run by tests/test_binding.py
// against mocc_interface.hpp; in a MOCC tree the same class includes MOCC's
// own headers and is selected by TransportSweeperFactory
// (src/sweepers/transport_sweeper_factory.cpp:37-42).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "mocc_interface.hpp"
#include "mocgpu.h"

namespace mocc {
namespace moc {

class MoCSweeperGPU : public TransportSweeper {
  public:
    // The library reads the same XML input (and .xsl library text, or the
    // file its <material_lib path> names under base_dir) and traces the same
    // rays; precision -1 takes the input's <sweeper precision>.
    MoCSweeperGPU(const std::string &xml, const std::string &xsl, const std::string &base_dir, int precision = -1)
    {
        check(mocgpu_problem_create(xml.c_str(), xsl.empty() ? nullptr : xsl.c_str(), base_dir.c_str(), &problem_),
              __LINE__);
        int64_t sz[MOCGPU_SZ_COUNT];
        check(mocgpu_problem_sizes(problem_, sz), __LINE__);
        n_group_ = (int)sz[MOCGPU_SZ_NGROUP];
        n_reg_ = (int)sz[MOCGPU_SZ_NFSR];
        n_pin_ = (int)sz[MOCGPU_SZ_NPIN];
        nx_ = (int)sz[MOCGPU_SZ_NX];
        ny_ = (int)sz[MOCGPU_SZ_NY];
        n_surf_ = (int)sz[MOCGPU_SZ_NSURF];
        check(mocgpu_problem_options(problem_, &opts_), __LINE__);
        int rc = mocgpu_sweeper_create(problem_, precision, &gpu_);
        if (rc != MOCGPU_OK) {
            mocgpu_problem_destroy(problem_);
            check(rc, __LINE__);
        }
    }
    ~MoCSweeperGPU() override
    {
        mocgpu_sweeper_destroy(gpu_);
        mocgpu_problem_destroy(problem_);
    }
    MoCSweeperGPU(const MoCSweeperGPU &) = delete;
    MoCSweeperGPU &operator=(const MoCSweeperGPU &) = delete;

    const mocgpu_options &options() const { return opts_; }
    mocgpu_sweeper *handle() { return gpu_; }
    int n_reg() const override { return n_reg_; }
    int n_group() const override { return n_group_; }
    int n_pin() const { return n_pin_; }

    void initialize() override { check(mocgpu_initialize(gpu_), __LINE__); }
    // Source::initialize_group + fission + in_scatter (source.cpp:41-112) on
    // the device: what MOCC's FixedSourceSolver::step asks of the Source
    // before each group sweep (the binding's Source forwards here)
    void build_source(int group) { check(mocgpu_source_group(gpu_, group), __LINE__); }
    void sweep(int group) override { check(mocgpu_sweep_group(gpu_, group), __LINE__); }
    void calc_fission_source(real_t k, ArrayB1 &fs) const override
    {
        check(mocgpu_calc_fission_source(gpu_, k, fs.size() ? fs.data() : nullptr), __LINE__);
    }
    real_t total_fission(bool old) const override
    {
        double v = 0.0;
        check(mocgpu_total_fission(gpu_, old ? 1 : 0, &v), __LINE__);
        return v;
    }
    void store_old_flux() override { check(mocgpu_store_old_flux(gpu_), __LINE__); }
    real_t flux_residual() const override
    {
        double r = 0.0;
        check(mocgpu_flux_residual(gpu_, &r), __LINE__);
        return r;
    }
    // MoCSweeper's pin mesh in 2-D: PIN and PIN_PLANE are the same mesh
    void get_pin_flux_1g(int g, ArrayB1 &flux, MeshTreatment t = MeshTreatment::PIN) const override
    {
        pin_mesh_only(t);
        check(mocgpu_get_pin_flux_1g(gpu_, g, flux.data()), __LINE__);
    }
    real_t set_pin_flux_1g(int g, const ArrayB1 &flux, MeshTreatment t = MeshTreatment::PIN) override
    {
        pin_mesh_only(t);
        double r = 0.0;
        check(mocgpu_set_pin_flux_1g(gpu_, g, flux.data(), &r), __LINE__);
        return r;
    }
    ArrayB3 pin_powers() const override
    {
        ArrayB3 p(1, ny_, nx_);
        check(mocgpu_pin_powers(gpu_, p.data()), __LINE__);
        return p;
    }
    void set_coarse_data(CoarseData *cd) override
    {
        TransportSweeper::set_coarse_data(cd);
        check(mocgpu_set_coarse_data(gpu_, cd != nullptr), __LINE__);
    }
    // device homogenisation of the current flux, one region per pin
    // (coarse-cell order): what MOCC's CMFD builds its operator from
    SP_XSMeshHomogenized_t get_homogenized_xsmesh() override
    {
        auto x = std::make_shared<XSMeshHomogenized>();
        const size_t n = (size_t)n_pin_ * n_group_;
        x->xstr.resize(n);
        x->xsnf.resize(n);
        x->xsf.resize(n);
        x->xsch.resize(n);
        x->xsrm.resize(n);
        x->xssc.resize(n * n_group_);
        check(mocgpu_homogenized_xs(gpu_, x->xstr.data(), x->xsnf.data(), x->xsf.data(), x->xsch.data(),
                                    x->xsrm.data(), x->xssc.data()),
              __LINE__);
        return x;
    }
    // MoCSweeper::update_incoming_flux (moc_sweeper.cpp:255-291) from the
    // partial currents MOCC's CMFD stored in CoarseData (CMFD::store_currents,
    // cmfd.cpp:555-638); MOCC's lookup (mode 1)
    void update_incoming_flux() override
    {
        if (!coarse_data_) return;
        const CoarseData &cd = *coarse_data_;
        std::vector<double> part((size_t)n_group_ * n_surf_), old(part.size());
        for (int g = 0; g < n_group_; g++)
            for (int is = 0; is < n_surf_; is++) {
                const auto &p = cd.partial_current[(size_t)is * n_group_ + g];
                part[(size_t)g * n_surf_ + is] = 2.0 * (p[0] + p[1]);
                if (cd.has_old_partial()) {
                    const auto &q = cd.partial_current_old[(size_t)is * n_group_ + g];
                    old[(size_t)g * n_surf_ + is] = 2.0 * (q[0] + q[1]);
                }
            }
        check(mocgpu_update_incoming_flux(gpu_, part.data(), cd.has_old_partial() ? old.data() : nullptr,
                                          cd.has_old_partial() ? 1 : 0, 1),
              __LINE__);
    }
    // MoCSweeper::apply_transverse_leakage (moc_sweeper.cpp:435-472), which
    // MOCC's 2-D/3-D sweeper calls between building a group's source and
    // sweeping it; tl is [n_reg], splitting as <sweeper tl_splitting> says
    void apply_transverse_leakage(int group, const ArrayB1 &tl)
    {
        check(mocgpu_apply_transverse_leakage(gpu_, group, tl.data()), __LINE__);
    }
    // EigenSolver::do_cmfd (eigen_solver.cpp:263-291) in one call: coarse
    // flux, homogenisation, CMFD::solve and the fine-flux rescale on the device
    void cmfd(real_t &k) { check(mocgpu_cmfd_solve(gpu_, &k), __LINE__); }

  private:
    static void check(int rc, int line)
    {
        if (rc != MOCGPU_OK) throw Exception(__FILE__, line, "MoCSweeperGPU", mocgpu_last_error());
    }
    static void pin_mesh_only(MeshTreatment t)
    {
        if (t != MeshTreatment::PIN && t != MeshTreatment::PIN_PLANE)
            throw Exception(__FILE__, __LINE__, "MoCSweeperGPU", "only the pin mesh (PIN, PIN_PLANE) is supported");
    }
    mocgpu_problem *problem_ = nullptr;
    mocgpu_sweeper *gpu_ = nullptr;
    mocgpu_options opts_{};
    int n_group_ = 0, n_reg_ = 0, n_pin_ = 0, nx_ = 0, ny_ = 0, n_surf_ = 0;
};

} // namespace moc
} // namespace mocc
