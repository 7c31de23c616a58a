// A stand-in for the parts of MOCC's headers that a GPU sweeper binding
// needs: the TransportSweeper interface (src/core/transport_sweeper.hpp:41-351),
// MeshTreatment (src/core/mesh.hpp:37-48), the 1-D/2-D/3-D real arrays the
// interface passes (MOCC uses Blitz++ arrays; plain contiguous row-major
// storage here) and the partial-current store of CoarseData
// (src/core/coarse_data.hpp:35-166). Written for this repository so that the
// binding in moc_sweeper_gpu.hpp compiles and runs without a MOCC build; a
// MOCC build includes MOCC's own headers instead.
#pragma once

#include <array>
#include <memory>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

namespace mocc {

using real_t = double;

enum class MeshTreatment : unsigned char { TRUE, PIN, PLANE, PIN_PLANE };

// Contiguous row-major arrays (the last index fastest, as in MOCC's ArrayB2
// flux_(n_reg, n_group)).
struct ArrayB1 {
    std::vector<real_t> v;
    explicit ArrayB1(std::size_t n = 0) : v(n, 0.0) {}
    real_t *data() { return v.data(); }
    const real_t *data() const { return v.data(); }
    std::size_t size() const { return v.size(); }
    real_t &operator()(std::size_t i) { return v[i]; }
    real_t operator()(std::size_t i) const { return v[i]; }
};
struct ArrayB2 {
    std::size_t n0 = 0, n1 = 0;
    std::vector<real_t> v;
    ArrayB2(std::size_t a = 0, std::size_t b = 0) : n0(a), n1(b), v(a * b, 0.0) {}
    real_t *data() { return v.data(); }
    const real_t *data() const { return v.data(); }
    real_t &operator()(std::size_t i, std::size_t j) { return v[i * n1 + j]; }
    real_t operator()(std::size_t i, std::size_t j) const { return v[i * n1 + j]; }
};
struct ArrayB3 {
    std::size_t n0 = 0, n1 = 0, n2 = 0;
    std::vector<real_t> v;
    ArrayB3(std::size_t a = 0, std::size_t b = 0, std::size_t c = 0) : n0(a), n1(b), n2(c), v(a * b * c, 0.0) {}
    real_t *data() { return v.data(); }
    real_t operator()(std::size_t i, std::size_t j, std::size_t k) const { return v[(i * n1 + j) * n2 + k]; }
};

// MOCC's Exception carries the file, line and function of the EXCEPT site.
struct Exception : std::runtime_error {
    Exception(const char *file, int line, const char *func, const std::string &msg)
        : std::runtime_error(std::string(file) + ":" + std::to_string(line) + " (" + func + "): " + msg)
    {
    }
};

// The partial currents CMFD::store_currents leaves for
// MoCSweeper::update_incoming_flux: [surface][group] pairs (J+, J-), the
// previous solve's copy and whether it exists.
struct CoarseData {
    int n_surf = 0, n_group = 0;
    std::vector<std::array<real_t, 2>> partial_current, partial_current_old;
    bool has_old_partial_ = false;
    bool has_old_partial() const { return has_old_partial_; }
};

// Homogenised cross sections per pin (what get_homogenized_xsmesh hands to
// CMFD): [n_pin][G], scattering [n_pin][G][G].
struct XSMeshHomogenized {
    std::vector<real_t> xstr, xsnf, xsf, xsch, xsrm, xssc;
};
using SP_XSMeshHomogenized_t = std::shared_ptr<XSMeshHomogenized>;

// MOCC's TransportSweeper: the duties an eigenvalue driver calls.
class TransportSweeper {
  public:
    virtual ~TransportSweeper() = default;
    virtual void sweep(int group) = 0;
    virtual void initialize() = 0;
    virtual void update_incoming_flux() = 0;
    virtual void get_pin_flux_1g(int group, ArrayB1 &flux, MeshTreatment treatment = MeshTreatment::PIN) const = 0;
    virtual real_t set_pin_flux_1g(int group, const ArrayB1 &pin_flux, MeshTreatment treatment = MeshTreatment::PIN) = 0;
    virtual SP_XSMeshHomogenized_t get_homogenized_xsmesh() = 0;
    virtual void calc_fission_source(real_t k, ArrayB1 &fission_source) const = 0;
    virtual void store_old_flux() = 0;
    virtual real_t flux_residual() const = 0;
    virtual real_t total_fission(bool old = false) const = 0;
    virtual ArrayB3 pin_powers() const = 0;
    virtual void set_coarse_data(CoarseData *cd) { coarse_data_ = cd; }
    virtual int n_reg() const = 0;
    virtual int n_group() const = 0;

  protected:
    CoarseData *coarse_data_ = nullptr;
};

} // namespace mocc
