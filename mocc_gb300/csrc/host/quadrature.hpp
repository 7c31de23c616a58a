// Angular quadratures for the 2-D MoC path.
//
// Follows MOCC's AngularQuadrature (src/core/angular_quadrature.cpp:47-113,
// 288-352; product sets src/core/product_quadrature.hpp:32-164; level
// symmetric src/core/level_symmetric.hpp). Angles are stored octant-major
// (8 octants); within an octant a product set is azimuth-major then polar.
#pragma once

#include <vector>

#include "geom.hpp"

namespace mocgpu {

struct XmlNode;

enum class QuadType { LS, CHEB_GAUSS, CHEB_YAMAMOTO, USER };

struct AngularQuadrature {
    QuadType type = QuadType::CHEB_YAMAMOTO;
    int n_azimuthal = -1; // per octant
    int n_polar = -1;
    int ndir_oct = 0;
    std::vector<Angle> angles; // 8 * ndir_oct

    static AngularQuadrature from_xml(const XmlNode &node);
    static AngularQuadrature chebyshev_yamamoto(int n_azi, int n_pol);

    int ndir() const { return (int)angles.size(); }
    const Angle &operator[](int i) const { return angles[i]; }

    // Octant (0-based) reflection table: reflect across X, Y, Z normals.
    int reflect(int iang, Normal n) const
    {
        static const int table[3][8] = {{1, 0, 3, 2, 5, 4, 7, 6}, {3, 2, 1, 0, 7, 6, 5, 4}, {4, 5, 6, 7, 0, 1, 2, 3}};
        int oct = iang / ndir_oct;
        return iang + (table[(int)n][oct] - oct) * ndir_oct;
    }
    // 2-D reverse: the opposite direction within the upper hemisphere.
    int reverse(int iang) const { return (iang + ndir_oct * 2) % (ndir_oct * 4); }

    void modify_angle(int iang, const Angle &a);
    void update_weights(); // Chebyshev azimuthal weights after modularisation

    // Number of distinct track sets per octant and polar angles per set.
    bool is_product() const { return type == QuadType::CHEB_GAUSS || type == QuadType::CHEB_YAMAMOTO; }
    int polars_per_set() const { return is_product() ? n_polar : 1; }
};

std::vector<std::pair<double, double>> gen_yamamoto(int n_polar);
std::vector<std::pair<double, double>> gen_chebyshev(int n_azi);
std::vector<std::pair<double, double>> gen_gauss(int n_polar);

} // namespace mocgpu
