#include "quadrature.hpp"

#include <algorithm>
#include <cmath>

#include "xml.hpp"

namespace mocgpu {

std::vector<std::pair<double, double>> gen_yamamoto(int n_polar)
{
    // Tabuchi-Yamamoto optimal 3-point polar set (published values).
    if (n_polar != 3) MOCGPU_THROW(1, "Yamamoto quadrature supports n_polar=3 only");
    return {{0.167429147795000, 4.623300000000000E-002},
            {0.567715121084000, 0.283619000000000},
            {1.20253314678900, 0.670148000000000}};
}

std::vector<std::pair<double, double>> gen_chebyshev(int n_azi)
{
    std::vector<std::pair<double, double>> v;
    double w = 1.0 / n_azi;
    double d = 0.5 * kPi / (2 * n_azi);
    for (int i = 0; i < n_azi; i++) v.emplace_back(d * (2 * i + 1), w);
    return v;
}

// Gauss-Legendre on [-1, 1] with 2*n_polar points; the n_polar positive
// cosines are returned as polar angles (largest angle first) with weights
// normalised to one over the half range.
std::vector<std::pair<double, double>> gen_gauss(int n_polar)
{
    const int N = 2 * n_polar;
    std::vector<double> x(N), w(N);
    for (int i = 0; i < N; i++) {
        double z = std::cos(kPi * (i + 0.75) / (N + 0.5));
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= N; k++) {
                double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = pk;
            }
            double dp = N * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) {
                // final derivative for the weight
                p0 = 1.0;
                p1 = z;
                for (int k = 2; k <= N; k++) {
                    double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                    p0 = p1;
                    p1 = pk;
                }
                dp = N * (z * p1 - p0) / (z * z - 1.0);
                break;
            }
        }
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= N; k++) {
            double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = pk;
        }
        double dp = N * (z * p1 - p0) / (z * z - 1.0);
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
    std::vector<std::pair<double, double>> out;
    std::vector<std::pair<double, double>> pos;
    for (int i = 0; i < N; i++)
        if (x[i] > 0.0) pos.emplace_back(x[i], w[i]);
    // ascending cosine == descending polar angle
    std::sort(pos.begin(), pos.end());
    double ws = 0.0;
    for (auto &p : pos) ws += p.second;
    for (auto &p : pos) out.emplace_back(std::acos(p.first), p.second / ws);
    return out;
}

namespace {
std::vector<Angle> gen_product(const std::vector<std::pair<double, double>> &azi,
                               const std::vector<std::pair<double, double>> &pol)
{
    std::vector<Angle> a;
    double wsum = 0.0;
    for (const auto &az : azi)
        for (const auto &p : pol) {
            a.emplace_back(Direction::from_angles(az.first, p.first), az.second * p.second);
            wsum += az.second * p.second;
        }
    for (auto &x : a) x.weight /= wsum;
    return a;
}

// Level-symmetric S_N sets for N <= 8 (published Lewis & Miller tables).
std::vector<Angle> gen_level_symmetric(int order)
{
    if (order % 2 != 0 || order < 2 || order > 8) MOCGPU_THROW(1, "level-symmetric order must be 2, 4, 6 or 8");
    static const double mu0[] = {0.577350269189626, 0.350021000000000, 0.266636000000000, 0.218218218218218};
    static const std::vector<std::vector<double>> wts = {
        {1.0}, {1.0 / 3.0}, {0.1761262, 0.1572071}, {0.1209876, 0.0907408, 0.0925925}};
    static const std::vector<std::vector<int>> maps = {
        {1}, {1, 1, 1}, {1, 2, 2, 1, 2, 1}, {1, 2, 2, 2, 3, 2, 1, 2, 2, 1}};
    const int n = order / 2;
    std::vector<double> mu{mu0[n - 1]};
    if (order > 2) {
        double dmu = 2.0 * (1.0 - 3.0 * mu[0] * mu[0]) / (double)(order - 2);
        for (int i = 1; i < n; i++) mu.push_back(std::sqrt(mu[0] * mu[0] + i * dmu));
    }
    std::vector<Angle> a;
    double wsum = 0.0;
    int k = 0;
    for (int i = 0; i < n; i++)
        for (int j = 0; j <= i; j++) {
            a.emplace_back(Direction::from_cosines(mu[i - j], mu[j], mu[n - i - 1]), wts[n - 1][maps[n - 1][k] - 1]);
            wsum += a.back().weight;
            k++;
        }
    for (auto &x : a) x.weight /= wsum;
    return a;
}

void expand_octants(std::vector<Angle> &a, int ndir_oct)
{
    a.resize(ndir_oct);
    for (int oct = 2; oct <= 8; oct++)
        for (int i = 0; i < ndir_oct; i++) a.push_back(a[i].to_octant(oct));
}
} // namespace

AngularQuadrature AngularQuadrature::chebyshev_yamamoto(int n_azi, int n_pol)
{
    AngularQuadrature q;
    q.type = QuadType::CHEB_YAMAMOTO;
    q.n_azimuthal = n_azi;
    q.n_polar = n_pol;
    q.angles = gen_product(gen_chebyshev(n_azi), gen_yamamoto(n_pol));
    q.ndir_oct = (int)q.angles.size();
    expand_octants(q.angles, q.ndir_oct);
    return q;
}

AngularQuadrature AngularQuadrature::from_xml(const XmlNode &node)
{
    AngularQuadrature q;
    q.n_azimuthal = node.attr_int("n_azimuthal", -1);
    q.n_polar = node.attr_int("n_polar", -1);
    std::string t = sanitize(node.attr("type"));
    if (t == "ls" || t == "level-symmetric") {
        q.type = QuadType::LS;
        q.angles = gen_level_symmetric(node.attr_int("order", -1));
    } else if (t == "cg" || t == "chebyshev-gauss") {
        if (q.n_azimuthal < 1 || q.n_polar < 1) MOCGPU_THROW(1, "Number of polar or azimuthal angles is invalid");
        q.type = QuadType::CHEB_GAUSS;
        q.angles = gen_product(gen_chebyshev(q.n_azimuthal), gen_gauss(q.n_polar));
    } else if (t == "cy" || t == "chebyshev-yamamoto") {
        if (q.n_azimuthal < 1 || q.n_polar < 1) MOCGPU_THROW(1, "Number of polar or azimuthal angles is invalid");
        q.type = QuadType::CHEB_YAMAMOTO;
        q.angles = gen_product(gen_chebyshev(q.n_azimuthal), gen_yamamoto(q.n_polar));
    } else if (t == "user") {
        q.type = QuadType::USER;
        for (const XmlNode *an : node.children_named("angle")) {
            double w = an->attr_double("weight", 0.0);
            if (w <= 0.0) MOCGPU_THROW(1, "Invalid angle weight specified.");
            if (an->has_attr("ox"))
                q.angles.emplace_back(Direction::from_cosines(an->attr_double("ox", 2.0), an->attr_double("oy", 2.0),
                                                              an->attr_double("oz", 2.0)),
                                      w);
            else
                q.angles.emplace_back(Direction::from_angles(an->attr_double("alpha", 0.0), an->attr_double("theta", 0.0)), w);
        }
        if (q.angles.empty()) MOCGPU_THROW(1, "user quadrature without angles");
    } else {
        MOCGPU_THROW(1, "Invalid angular quadrature type specified: " + t);
    }
    q.ndir_oct = (int)q.angles.size();
    expand_octants(q.angles, q.ndir_oct);
    return q;
}

void AngularQuadrature::modify_angle(int iang, const Angle &a)
{
    angles[iang] = a;
    for (int oct = 1; oct < 8; oct++) angles[iang + oct * ndir_oct] = a.to_octant(oct + 1);
}

void AngularQuadrature::update_weights()
{
    if (!is_product()) return; // LS and user sets keep their weights
    std::vector<std::pair<double, double>> pol =
        (type == QuadType::CHEB_GAUSS) ? gen_gauss(n_polar) : gen_yamamoto(n_polar);
    std::vector<double> azi;
    for (int i = 0; i < ndir_oct; i++) azi.push_back(angles[i].alpha);
    std::sort(azi.begin(), azi.end());
    azi.erase(std::unique(azi.begin(), azi.end(), fp_equiv_ulp), azi.end());
    if ((int)azi.size() != n_azimuthal) MOCGPU_THROW(1, "Wrong number of azimuthal angles!");
    std::vector<double> bounds{0.0};
    for (int i = 0; i < n_azimuthal - 1; i++) bounds.push_back((azi[i] + azi[i + 1]) / 2.0);
    bounds.push_back(kHalfPi);
    std::vector<std::pair<double, double>> pairs;
    for (int i = 0; i < n_azimuthal; i++) pairs.emplace_back(azi[i], (bounds[i + 1] - bounds[i]) / kHalfPi);
    angles = gen_product(pairs, pol);
    expand_octants(angles, ndir_oct);
}

} // namespace mocgpu
