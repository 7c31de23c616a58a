// Macroscopic cross-section library.
//
// Follows MOCC's material model:
//   .xsl reader                    src/core/material_lib.cpp:45-149
//   Material (chi normalisation,
//     sigma_tr = sigma_a + out-scatter) src/core/material.cpp:22-62
//   scattering rows "to" x "from"  src/core/scattering_matrix.cpp:57-123
// plus a seeded synthetic-library generator for the benchmark workloads
// (log-uniform total XS, downscatter-dominant scattering with small upscatter
// into the last groups, fissile materials only in fuel).
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace mocgpu {

struct Material {
    std::string name;
    int ng = 0;
    std::vector<double> xsab, xsnf, xsf, xsch, xstr;
    std::vector<double> scat; // dense [to][from], ng*ng
    std::vector<double> out;  // total out-scatter from each group
    bool fissile = false;

    double s(int to, int from) const { return scat[(size_t)to * ng + from]; }
    // Builds derived fields (chi normalisation, out-scatter, sigma_tr).
    void finalize();
};

struct MaterialLib {
    int ng = 0;
    std::vector<double> group_bounds;
    std::vector<Material> lib;            // library order
    std::map<std::string, int> by_name;   // name -> library index
    std::map<int, int> id_to_dense;       // user id -> dense index
    std::vector<Material> assigned;       // dense order (assignment order)

    static MaterialLib from_xsl_text(const std::string &text);
    void assign(int id, const std::string &name);
    const Material &by_id(int id) const;
    bool has(int id) const { return id_to_dense.count(id) > 0; }
};

// Parameters of the synthetic library (all materials share ng).
struct SyntheticXsSpec {
    int ng = 7;
    uint64_t seed = 1;
    int n_fuel = 3;                  // fuel compositions fuel1..fuelN
    std::vector<double> fuel_nf_scale; // nu-fission scale per fuel composition
    double mod_factor = 1.0;         // multiplies moderator sigma_t and scattering
    double fuel_nf_factor = 1.0;     // multiplies every fuel nu-fission
};

// Emits a library in .xsl text form. Materials: fuel1..fuelN, moderator.
std::string synthetic_xsl(const SyntheticXsSpec &spec);

} // namespace mocgpu
