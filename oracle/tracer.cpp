/*
 * CPU oracle: MOCC's XML input, cross-section library, core mesh, angular
 * quadrature and modular ray tracer, restated so that the oracle builds its
 * problem from the input text alone.
 *
 * TEST INFRASTRUCTURE ONLY: the checker's own path from input to the flat
 * problem (orc_problem) its solver consumes. No product code path links,
 * loads or calls it, and it links nothing of the product.
 *
 * Restated MOCC routines (paths within the MOCC repository):
 *   fuzzy comparisons          src/util/fp_utils.hpp
 *   Point2, Line/Circle/Box    src/core/geometry/points.hpp, geom.hpp, box.cpp
 *   Direction, Angle           src/core/geometry/direction.hpp, angle.cpp
 *   rational approximation     src/util/rational_approximation.hpp:39-80
 *   Sn / product quadratures   src/core/level_symmetric.hpp,
 *                              src/core/product_quadrature.hpp,
 *                              src/core/angular_quadrature.cpp:47-113, 288-352
 *   material library           src/core/material_lib.cpp, material.cpp,
 *                              scattering_matrix.cpp
 *   pin meshes                 src/core/pin_mesh_cyl.cpp:36-311,
 *                              src/core/pin_mesh_rect.cpp
 *   pins, lattices, assemblies,
 *   core and plane lookup      src/core/pin.cpp, lattice.cpp, assembly.cpp,
 *                              core.cpp, plane.cpp, core_mesh.cpp
 *   mesh trace and surfaces    src/core/mesh.cpp:88-600
 *   ray laydown (core or pin
 *   modularity, rational or
 *   trig modularisation),
 *   trace, volume correction
 *   (flat, angle, none)        src/sweepers/moc/ray_data.cpp:67-527,
 *                              src/sweepers/moc/ray.cpp:52-175
 *   solver options             src/solvers/eigen_solver.cpp, src/core/cmfd.cpp,
 *                              src/sweepers/moc/moc_sweeper.cpp
 *
 * Two rules differ from MOCC on purpose, the same way in the library this
 * oracle checks: (1) the coarse walk of a ray takes the surfaces between two
 * pin crossings from the cells of the traced segments (a crossing shorter
 * than 1e-9 cm, a ray grazing a pin-cell corner, is folded into its
 * neighbour; diagonal neighbours cross the x face and then the y face; a
 * pin-line crossing within 1e-10 cm of a ray's end point is dropped), where
 * MOCC's fuzzy point tests at a corner can name a surface off the ray's path
 * and break the pin-cell neutron balance that CMFD needs;
 * (2) the vertical mesh lines of the core trace span the larger of the core
 * width and height (MOCC uses the width; the same for square cores).
 * With mocc_literal set, orc_trace keeps MOCC's own behaviour for (1): every
 * pin-line crossing is kept and the coarse data comes from the fuzzy point
 * tests at the crossing points (ray.cpp:84-166), so tests can show where
 * the two differ.
 * Tracks of one azimuth are stored once for all its polar angles (MOCC
 * traces the identical rays once per polar angle).
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "oracle.h"

namespace trc {

using std::string;
using std::vector;

struct Fail : std::runtime_error {
    explicit Fail(const string &m) : std::runtime_error(m) {}
};

constexpr double PI = 3.1415926535897932;
constexpr double TWOPI = 2.0 * PI;
constexpr double HPI = 0.5 * PI;
constexpr double FUZZ = 200 * std::numeric_limits<double>::epsilon();

// ---- fp_utils.hpp ------------------------------------------------------------
bool eq_ulp(double a, double b)
{
    int64_t ia, ib;
    std::memcpy(&ia, &a, 8);
    std::memcpy(&ib, &b, 8);
    if (ia < 0) ia = 0x80000000LL - ia;
    if (ib < 0) ib = 0x80000000LL - ib;
    return std::llabs(ia - ib) < 200;
}
bool eq_abs(double a, double b) { return std::fabs(a - b) < FUZZ; }
bool eq_rel(double a, double b) { return std::fabs(a - b) / std::fabs(a) < FUZZ; }
bool eq(double a, double b)
{
    if (eq_abs(a, b)) return true;
    if ((a < 0.0) != (b < 0.0)) return false;
    return eq_ulp(a, b);
}
bool fuzzy_lt(double l, double r) { return (l - r) / std::fabs(r) < -FUZZ; }

// ---- geometry -------------------------------------------------------------------
struct Pt {
    double x = 0, y = 0;
    bool ok = false;
    Pt() = default;
    Pt(double a, double b) : x(a), y(b), ok(true) {}
};
double dist(const Pt &a, const Pt &b) { return std::sqrt((a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y)); }
Pt mid(const Pt &a, const Pt &b) { return Pt(0.5 * (a.x + b.x), 0.5 * (a.y + b.y)); }
double alpha_of(const Pt &p) { return (p.y > 0.0) ? std::atan2(p.y, p.x) : std::atan2(p.y, p.x) + TWOPI; }
struct Seg {
    Pt a, b;
};
// points sorted by y (rays run upward), fuzzy duplicates removed
void sort_unique(vector<Pt> &ps)
{
    std::sort(ps.begin(), ps.end(), [](const Pt &p, const Pt &q) { return p.y < q.y; });
    ps.erase(std::unique(ps.begin(), ps.end(), [](const Pt &p, const Pt &q) { return eq(p.x, q.x) && eq(p.y, q.y); }),
             ps.end());
}
// geom.hpp Intersect(Line, Line)
int cross_lines(const Seg &l1, const Seg &l2, Pt &p)
{
    double u1 = l1.b.x - l1.a.x, u2 = l1.b.y - l1.a.y;
    double v1 = l2.b.x - l2.a.x, v2 = l2.b.y - l2.a.y;
    double w1 = l1.a.x - l2.a.x, w2 = l1.a.y - l2.a.y;
    double d = u1 * v2 - u2 * v1;
    double s = v1 * w2 - v2 * w1;
    double t = u1 * w2 - u2 * w1;
    s = s / d;
    t = t / d;
    if ((0.0 <= s) & (s <= 1.0) & (0.0 <= t) & (t <= 1.0)) {
        p = Pt(l1.a.x + s * u1, l1.a.y + s * u2);
        return 1;
    }
    return 0;
}
// geom.hpp Intersect(Line, Circle) for a circle at the origin
int cross_circle(const Seg &l, double r, Pt &p1, Pt &p2)
{
    double u1 = l.b.x - l.a.x, u2 = l.b.y - l.a.y;
    double w1 = l.a.x, w2 = l.a.y;
    double b = w1 * u1 + w2 * u2;
    double c = w1 * w1 + w2 * w2 - r * r;
    if ((c > 0.0) & (b > 0.0)) return 0;
    double a = u1 * u1 + u2 * u2;
    double disc = b * b - a * c;
    if (disc < 0.0) return 0;
    if (eq_rel(disc, 0.0)) return 0;
    double ra = 1.0 / a;
    disc = std::sqrt(disc);
    double t1 = (-b - disc) * ra, t2 = (-b + disc) * ra;
    int n = 0;
    if ((0.0 < t1) & (t1 < 1.0)) {
        p1 = Pt(l.a.x + u1 * t1, l.a.y + u2 * t1);
        n++;
    }
    if ((0.0 < t2) & (t2 < 1.0)) {
        Pt q(l.a.x + u1 * t2, l.a.y + u2 * t2);
        if (n == 0) p1 = q;
        else p2 = q;
        n++;
    }
    return n;
}
// box.cpp Box::intersect: where a ray from p at azimuth alpha leaves [lo, hi]
Pt box_exit(Pt lo, Pt hi, Pt p, double alpha)
{
    double ox = std::cos(alpha), oy = std::sin(alpha);
    double dmin = 1.0e12, d, x, y;
    Pt out;
    x = lo.x;
    d = (lo.x - p.x) / ox;
    y = p.y + oy * d;
    if ((std::fabs(d) > FUZZ) && (d < dmin) && (y > lo.y) && (y < hi.y)) {
        dmin = std::fabs(d);
        out = Pt(x, y);
    }
    x = hi.x;
    d = (hi.x - p.x) / ox;
    y = p.y + oy * d;
    if ((std::fabs(d) > FUZZ) && (d < dmin) && (y > lo.y) && (y < hi.y)) {
        dmin = std::fabs(d);
        out = Pt(x, y);
    }
    y = lo.y;
    d = (lo.y - p.y) / oy;
    x = p.x + ox * d;
    if ((std::fabs(d) > FUZZ) && (d < dmin) && (x > lo.x) && (x < hi.x)) {
        dmin = std::fabs(d);
        out = Pt(x, y);
    }
    y = hi.y;
    d = (hi.y - p.y) / oy;
    x = p.x + ox * d;
    if ((std::fabs(d) > FUZZ) && (d < dmin) && (x > lo.x) && (x < hi.x)) {
        dmin = std::fabs(d);
        out = Pt(x, y);
    }
    return out;
}

// ---- direction.hpp / angle.cpp --------------------------------------------------
struct Ang {
    double ox, oy, oz, alpha, theta, rsin, w;
};
Ang ang_from_at(double alpha, double theta, double w)
{
    Ang a;
    a.alpha = alpha;
    a.theta = theta;
    a.ox = std::sin((long double)theta) * std::cos((long double)alpha);
    a.oy = std::sin((long double)theta) * std::sin((long double)alpha);
    a.oz = std::cos((long double)theta);
    a.rsin = 1.0 / std::sin((long double)theta);
    a.w = w;
    return a;
}
Ang ang_from_cos(double ox, double oy, double oz, double w)
{
    Ang a;
    a.ox = ox;
    a.oy = oy;
    a.oz = oz;
    long double oxb = ox, ozb = oz;
    long double th = std::acos(ozb);
    a.theta = th;
    a.alpha = std::acos(oxb / std::sin(th));
    if (oy < 0.0) a.alpha = TWOPI - a.alpha;
    a.rsin = 1.0l / std::sin(th);
    a.w = w;
    return a;
}
Ang to_octant(const Ang &a, int oct)
{
    const double x = std::fabs(a.ox), y = std::fabs(a.oy), z = std::fabs(a.oz);
    switch (oct) {
    case 1: return ang_from_cos(x, y, z, a.w);
    case 2: return ang_from_cos(-x, y, z, a.w);
    case 3: return ang_from_cos(-x, -y, z, a.w);
    case 4: return ang_from_cos(x, -y, z, a.w);
    case 5: return ang_from_cos(x, y, -z, a.w);
    case 6: return ang_from_cos(-x, y, -z, a.w);
    case 7: return ang_from_cos(-x, -y, -z, a.w);
    default: return ang_from_cos(x, -y, -z, a.w);
    }
}

// ---- quadratures ------------------------------------------------------------------
using Pairs = vector<std::pair<double, double>>;
Pairs yamamoto(int n)
{
    if (n != 3) throw Fail("Only support Yamamoto quadrature when npol=3");
    return {{0.167429147795000, 4.623300000000000E-002}, {0.567715121084000, 0.283619000000000},
            {1.20253314678900, 0.670148000000000}};
}
Pairs chebyshev(int n)
{
    Pairs v;
    double w = 1.0 / n, d = 0.5 * PI / (2 * n);
    for (int i = 0; i < n; i++) v.emplace_back(d * (2 * i + 1), w);
    return v;
}
// Gauss-Legendre polar angles in (0, pi/2) by Newton iteration on the
// Legendre polynomial of order 2 n (product_quadrature.hpp GenGauss)
Pairs gauss(int np)
{
    const int N = 2 * np - 1, N1 = 2 * np, N2 = 2 * np + 1;
    vector<double> xu(N1), y(N1), w(N1), y0(N1, 2.0), Lp(N1);
    vector<vector<double>> L(N1, vector<double>(N2));
    const double del = 2.0 / N;
    for (int i = 0; i < N1; i++) {
        xu[i] = -1.0 + i * del;
        y[i] = std::cos((2 * i + 1) * PI / (2 * N1)) + 0.27 / N1 * std::sin(PI * xu[i] * N / N2);
    }
    auto diff = [&]() {
        double m = 0.0;
        for (int i = 0; i < N1; i++) m = std::max(m, std::fabs(y[i] - y0[i]));
        return m;
    };
    while (diff() > FUZZ) {
        for (int m = 0; m < N1; m++) {
            L[m][0] = 1;
            L[m][1] = y[m];
        }
        for (int k = 1; k < N1; k++)
            for (int m = 0; m < N1; m++) L[m][k + 1] = ((2 * k + 1) * y[m] * L[m][k] - k * L[m][k - 1]) / (k + 1);
        for (int i = 0; i < N1; i++) Lp[i] = N2 * (L[i][N1 - 1] - y[i] * L[i][N2 - 1]) / (1 - y[i] * y[i]);
        y0 = y;
        for (int i = 0; i < N1; i++) y[i] = y0[i] - L[i][N2 - 1] / Lp[i];
    }
    for (int i = 0; i < N1; i++) w[i] = 1.0 / ((1 - y[i] * y[i]) * Lp[i] * Lp[i]) * N2 * N2 / (N1 * N1);
    for (auto &v : y) v = std::acos(v);
    for (int i = 0; i < np; i++) std::swap(y[i], y[N1 - 1 - i]);
    Pairs v;
    for (int i = np; i < N1; i++) v.emplace_back(y[i], w[i]);
    return v;
}
vector<Ang> product(const Pairs &azi, const Pairs &pol)
{
    vector<Ang> v;
    double ws = 0.0;
    for (auto &a : azi)
        for (auto &p : pol) {
            v.push_back(ang_from_at(a.first, p.first, a.second * p.second));
            ws += a.second * p.second;
        }
    for (auto &a : v) a.w /= ws;
    return v;
}
// level_symmetric.hpp GenSn: MOCC's tables of base cosines and weights
vector<Ang> level_symmetric(int order)
{
    static const double mu_base[] = {0.577350269189626, 0.350021000000000, 0.266636000000000, 0.218218218218218,
                                     0.192450089729876, 0.174077655955702, 0.161575000000000, 0.149071198499989};
    static const double w_unique[] = {1.0,       1.0 / 3.0, 0.1761262, 0.1572071, 0.1209876, 0.0907408, 0.0925925,
                                      0.0893043, 0.0725281, 0.0450455, 0.0539274, 0.0707734, 0.0558760, 0.0373436,
                                      0.0502654, 0.0258553, 0.0580031, 0.0488943, 0.0228095, 0.0393955, 0.0380920,
                                      0.0258382, 0.0082759, 0.0489967, 0.0413235, 0.0203158, 0.0265468, 0.0378883,
                                      0.0135404, 0.0326129, 0.0103825};
    static const int w_offset[] = {0, 1, 2, 4, 7, 11, 16, 23};
    static const int w_map[] = {1, 1, 1, 1, 1, 2, 2, 1, 2, 1, 1, 2, 2, 2, 3, 2, 1, 2, 2, 1, 1, 2, 2, 3, 4,
                                3, 2, 4, 4, 2, 1, 2, 3, 2, 1, 1, 2, 2, 3, 5, 3, 4, 6, 6, 4, 3, 6, 7, 6, 3,
                                2, 5, 6, 6, 5, 2, 1, 2, 3, 4, 3, 2, 1, 1, 2, 2, 3, 5, 3, 4, 6, 6, 4, 4, 7,
                                8, 7, 4, 3, 6, 8, 8, 6, 3, 2, 5, 6, 7, 6, 5, 2, 1, 2, 3, 4, 4, 3, 2, 1};
    static const int w_map_offset[] = {0, 1, 4, 10, 20, 35, 63};
    if (order % 2 != 0) throw Fail("Sn quadrature order must be even.");
    if (order < 2 || order > 14) throw Fail("Sn quadrature order out of the supported range");
    const int n = order / 2;
    vector<double> mu{mu_base[n - 1]};
    if (order > 2) {
        const double dmu = 2.0 * (1.0 - 3.0 * (mu[0] * mu[0])) / (double)(order - 2);
        for (int i = 1; i < n; i++) mu.push_back(std::sqrt(mu[0] * mu[0] + i * dmu));
    }
    const double *wts = &w_unique[w_offset[n - 1]];
    const int *map = &w_map[w_map_offset[n - 1]];
    vector<Ang> v;
    double ws = 0.0;
    int k = 0;
    for (int i = 0; i < n; i++)
        for (int j = 0; j <= i; j++) {
            v.push_back(ang_from_cos(mu[i - j], mu[j], mu[n - i - 1], wts[map[k] - 1]));
            ws += v.back().w;
            k++;
        }
    for (auto &a : v) a.w /= ws;
    return v;
}

enum QType { LS, CG, CY };
struct Quad {
    QType type;
    int n_azi = -1, n_pol = -1, ndir = 0;
    vector<Ang> ang; // 8 octants
    void expand()
    {
        ang.resize(ndir);
        for (int o = 2; o <= 8; o++)
            for (int i = 0; i < ndir; i++) ang.push_back(to_octant(ang[i], o));
    }
    void modify(int i, const Ang &a)
    {
        ang[i] = a;
        for (int o = 1; o < 8; o++) ang[i + o * ndir] = to_octant(a, o + 1);
    }
    // angular_quadrature.cpp:288-352: the azimuthal weights of a product
    // quadrature become the share of the quarter circle nearest each
    // modularised azimuth
    void update_weights()
    {
        if (type == LS) return;
        Pairs pol = (type == CG) ? gauss(n_pol) : yamamoto(n_pol);
        vector<double> az;
        for (int i = 0; i < ndir; i++) az.push_back(ang[i].alpha);
        std::sort(az.begin(), az.end());
        az.erase(std::unique(az.begin(), az.end(), eq_ulp), az.end());
        if ((int)az.size() != n_azi) throw Fail("Wrong number of azimuthal angles!");
        vector<double> b{0.0};
        for (int i = 0; i < n_azi - 1; i++) b.push_back((az[i] + az[i + 1]) / 2.0);
        b.push_back(HPI);
        Pairs ap;
        for (int i = 0; i < n_azi; i++) {
            double hpi = HPI;
            ap.emplace_back(az[i], (b[i + 1] - b[i]) / hpi);
        }
        ang = product(ap, pol);
        expand();
    }
};

// ---- minimal XML reader -------------------------------------------------------------
struct Node {
    string name, text;
    vector<std::pair<string, string>> attrs;
    vector<std::unique_ptr<Node>> kids;
    const Node *child(const string &n) const
    {
        for (auto &k : kids)
            if (k->name == n) return k.get();
        return nullptr;
    }
    vector<const Node *> children(const string &n) const
    {
        vector<const Node *> v;
        for (auto &k : kids)
            if (k->name == n) v.push_back(k.get());
        return v;
    }
    bool has(const string &a) const
    {
        for (auto &p : attrs)
            if (p.first == a) return true;
        return false;
    }
    string attr(const string &a, const string &d = "") const
    {
        for (auto &p : attrs)
            if (p.first == a) return p.second;
        return d;
    }
    double dbl(const string &a, double d) const
    {
        string s = attr(a);
        if (s.empty()) return d;
        char *e = nullptr;
        double v = std::strtod(s.c_str(), &e);
        return (e && e != s.c_str()) ? v : d;
    }
    int integer(const string &a, int d) const
    {
        string s = attr(a);
        if (s.empty()) return d;
        char *e = nullptr;
        long v = std::strtol(s.c_str(), &e, 10);
        return (e && e != s.c_str()) ? (int)v : d;
    }
    // pugixml's as_bool: true for a leading 1, t, T, y or Y
    bool boolean(const string &a, bool d) const
    {
        string s = attr(a);
        if (s.empty()) return d;
        char c = s[0];
        return c == '1' || c == 't' || c == 'T' || c == 'y' || c == 'Y';
    }
};
struct XmlReader {
    const string &s;
    size_t i = 0;
    explicit XmlReader(const string &t) : s(t) {}
    void skip_ws()
    {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
    }
    static string unescape(const string &t)
    {
        string o;
        for (size_t k = 0; k < t.size(); k++) {
            if (t[k] == '&') {
                size_t e = t.find(';', k);
                string ent = t.substr(k + 1, e - k - 1);
                if (ent == "lt") o += '<';
                else if (ent == "gt") o += '>';
                else if (ent == "amp") o += '&';
                else if (ent == "quot") o += '"';
                else if (ent == "apos") o += '\'';
                k = e;
            } else {
                o += t[k];
            }
        }
        return o;
    }
    // parses the children of `parent` until its closing tag (or the end)
    void parse_into(Node &parent)
    {
        while (i < s.size()) {
            size_t lt = s.find('<', i);
            if (lt == string::npos) {
                parent.text += unescape(s.substr(i));
                i = s.size();
                return;
            }
            parent.text += unescape(s.substr(i, lt - i));
            i = lt;
            if (s.compare(i, 4, "<!--") == 0) {
                size_t e = s.find("-->", i);
                if (e == string::npos) throw Fail("unterminated XML comment");
                i = e + 3;
            } else if (s.compare(i, 2, "<?") == 0) {
                size_t e = s.find("?>", i);
                if (e == string::npos) throw Fail("unterminated XML declaration");
                i = e + 2;
            } else if (s.compare(i, 2, "</") == 0) {
                size_t e = s.find('>', i);
                if (e == string::npos) throw Fail("unterminated closing tag");
                i = e + 1;
                return;
            } else {
                i++;
                auto n = std::make_unique<Node>();
                size_t b = i;
                while (i < s.size() && !std::isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') i++;
                n->name = s.substr(b, i - b);
                bool closed = false;
                while (true) {
                    skip_ws();
                    if (i >= s.size()) throw Fail("unterminated tag <" + n->name + ">");
                    if (s[i] == '/') {
                        closed = true;
                        i = s.find('>', i) + 1;
                        break;
                    }
                    if (s[i] == '>') {
                        i++;
                        break;
                    }
                    size_t a = i;
                    while (i < s.size() && s[i] != '=' && !std::isspace((unsigned char)s[i])) i++;
                    string an = s.substr(a, i - a);
                    skip_ws();
                    if (i >= s.size() || s[i] != '=') throw Fail("malformed attribute in <" + n->name + ">");
                    i++;
                    skip_ws();
                    char q = s[i++];
                    size_t e = s.find(q, i);
                    if (e == string::npos) throw Fail("unterminated attribute value");
                    n->attrs.emplace_back(an, unescape(s.substr(i, e - i)));
                    i = e + 1;
                }
                if (!closed) parse_into(*n);
                parent.kids.push_back(std::move(n));
            }
        }
    }
};
std::unique_ptr<Node> parse_xml(const string &text)
{
    auto root = std::make_unique<Node>();
    XmlReader r(text);
    r.parse_into(*root);
    return root;
}
template <typename T> vector<T> numbers(const string &t)
{
    vector<T> v;
    std::istringstream in(t);
    T x;
    while (in >> x) v.push_back(x);
    return v;
}
string lower(string s)
{
    for (auto &c : s) c = (char)std::tolower((unsigned char)c);
    // MOCC's sanitize also trims surrounding blanks
    size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == string::npos ? string() : s.substr(a, b - a + 1);
}

// ---- material library (material_lib.cpp) ------------------------------------------
struct Material {
    string name;
    vector<double> xstr, xsnf, xsf, xsch;
    vector<double> scat; // [to][from]
    bool fissile = false;
};
struct Library {
    int ng = 0;
    vector<double> bounds; // group upper energy bounds (material_lib.cpp:80-90)
    vector<Material> mats;
    std::map<string, int> by_name;
};
Library read_xsl(const string &text)
{
    // lines with '!' comments removed and blank lines skipped
    vector<string> lines;
    {
        std::istringstream in(text);
        string l;
        while (std::getline(in, l)) {
            size_t c = l.find('!');
            if (c != string::npos) l = l.substr(0, c);
            if (l.find_first_not_of(" \t\r") == string::npos) continue;
            lines.push_back(l);
        }
    }
    size_t li = 0;
    auto next = [&]() -> const string & {
        if (li >= lines.size()) throw Fail("cross-section library ends early");
        return lines[li++];
    };
    next(); // title
    Library lib;
    int nmat = 0;
    {
        std::istringstream in(next());
        if (!(in >> lib.ng >> nmat)) throw Fail("Failed to read number of groups!");
    }
    {
        std::istringstream in(next());
        for (int g = 0; g < lib.ng; g++) {
            double v;
            if (!(in >> v)) throw Fail("Trouble reading group bounds!");
            lib.bounds.push_back(v);
        }
    }
    const int G = lib.ng;
    for (int m = 0; m < nmat; m++) {
        std::istringstream head(next());
        string tag, name;
        head >> tag >> name;
        if (tag != "XSMACRO") throw Fail("expected XSMACRO in the cross-section library");
        Material mt;
        mt.name = name;
        vector<double> ab(G);
        mt.xsnf.resize(G);
        mt.xsf.resize(G);
        mt.xsch.resize(G);
        for (int g = 0; g < G; g++) {
            auto v = numbers<double>(next());
            if (v.size() != 4) throw Fail("Trouble reading XS data from library!");
            ab[g] = v[0];
            mt.xsnf[g] = v[1];
            mt.xsf[g] = v[2];
            mt.xsch[g] = v[3];
        }
        mt.scat.assign((size_t)G * G, 0.0);
        for (int to = 0; to < G; to++) {
            auto v = numbers<double>(next());
            if ((int)v.size() != G) throw Fail("Trouble reading scattering row");
            for (int from = 0; from < G; from++) mt.scat[(size_t)to * G + from] = v[from];
        }
        mt.fissile = std::any_of(mt.xsnf.begin(), mt.xsnf.end(), [](double v) { return v > 0.0; });
        if (std::any_of(mt.xsch.begin(), mt.xsch.end(), [](double v) { return v > 0.0; })) {
            double s = 0.0;
            for (double c : mt.xsch) s += c;
            for (double &c : mt.xsch) c /= s;
        }
        // transport = absorption + out-scatter; the out-scatter of group g
        // sums the banded rows that reach g (scattering_matrix.cpp:57-123)
        mt.xstr.resize(G);
        for (int g = 0; g < G; g++) {
            double out = 0.0;
            for (int to = 0; to < G; to++) {
                int lo = to, hi = to;
                for (int f = 0; f < G; f++)
                    if (mt.scat[(size_t)to * G + f] > 0.0) {
                        lo = std::min(lo, f);
                        break;
                    }
                for (int f = G - 1; f >= 0; f--)
                    if (mt.scat[(size_t)to * G + f] > 0.0) {
                        hi = std::max(hi, f);
                        break;
                    }
                if (g >= lo && g <= hi) out += mt.scat[(size_t)to * G + g];
            }
            mt.xstr[g] = ab[g] + out;
        }
        lib.by_name[name] = (int)lib.mats.size();
        lib.mats.push_back(mt);
    }
    return lib;
}

// ---- pin meshes ---------------------------------------------------------------------
struct PinMesh {
    bool cyl = true;
    double px = 0, py = 0;
    int n_xsreg = 0, n_reg = 0;
    // cylinder
    vector<double> radii;
    vector<int> sub_rad;
    int sub_azi = 0;
    vector<Seg> lines;
    // rectangle
    int nx = 0, ny = 0;
    vector<double> hx, hy;
    vector<double> areas;
    // FSRs of XS region x (rings carry sub_rad * sub_azi, the outer region sub_azi)
    int fsrs_of(int x) const
    {
        if (!cyl) return 1;
        return (x < (int)sub_rad.size()) ? sub_rad[x] * sub_azi : sub_azi;
    }
    int find_reg(Pt p) const
    {
        if (std::fabs(p.x) > 0.5 * px || std::fabs(p.y) > 0.5 * py) return -1;
        if (cyl) {
            double r = std::sqrt(p.x * p.x + p.y * p.y);
            unsigned ir = 0;
            for (ir = 0; ir < radii.size(); ir++)
                if (r < radii[ir]) break;
            int ia = (int)(alpha_of(p) / (TWOPI / sub_azi));
            return (int)ir * sub_azi + ia;
        }
        int ix = (int)(std::lower_bound(hx.begin(), hx.end(), p.x) - hx.begin()) - 1;
        int iy = (int)(std::lower_bound(hy.begin(), hy.end(), p.y) - hy.begin()) - 1;
        return nx * iy + ix;
    }
    // segments between p1 and p2 (pin-local), pin_mesh_cyl.cpp:177-219 /
    // pin_mesh_rect.cpp trace
    int trace(Pt p1, Pt p2, int first, vector<double> &len, vector<int> &reg) const
    {
        Seg l{p1, p2};
        vector<Pt> ps{p1, p2};
        if (cyl) {
            for (double r : radii) {
                Pt a, b;
                if (cross_circle(l, r, a, b) == 2) {
                    ps.push_back(a);
                    ps.push_back(b);
                }
            }
        }
        for (const Seg &li : lines) {
            Pt p;
            if (cross_lines(li, l, p) == 1) ps.push_back(p);
        }
        sort_unique(ps);
        for (size_t k = 1; k < ps.size(); k++) {
            len.push_back(dist(ps[k], ps[k - 1]));
            reg.push_back(find_reg(mid(ps[k], ps[k - 1])) + first);
        }
        return (int)ps.size() - 1;
    }
};
PinMesh read_mesh(const Node &n)
{
    PinMesh m;
    m.px = m.py = n.dbl("pitch", -1.0);
    if (m.px <= 0.0) throw Fail("Failed to read valid pin pitch.");
    string t = lower(n.attr("type"));
    if (t == "cyl") {
        m.cyl = true;
        const Node *r = n.child("radii");
        if (!r) throw Fail("cylindrical pin mesh without <radii>");
        vector<double> xr = numbers<double>(r->text);
        for (size_t i = 0; i + 1 < xr.size(); i++)
            if (xr[i] > xr[i + 1]) throw Fail("Pin radii do not appear to be ordered");
        if (xr.back() > m.px * 0.5) throw Fail("Largest radius is too big!");
        m.n_xsreg = (int)xr.size() + 1;
        const Node *sa = n.child("sub_azi");
        m.sub_azi = sa ? numbers<int>(sa->text).at(0) : 0;
        if (m.sub_azi % 2 != 0 || m.sub_azi > 8 || m.sub_azi < 2)
            throw Fail("Only supporting even azimuthal subdivisions <=8.");
        const Node *sr = n.child("sub_radii");
        m.sub_rad = sr ? numbers<int>(sr->text) : vector<int>();
        if ((int)m.sub_rad.size() != m.n_xsreg - 1) throw Fail("Wrong number of radial subdivisions specified.");
        // equal-area mesh rings within each cross-section ring
        double rxs = 0.0, ri = 0.0;
        for (int x = 0; x < m.n_xsreg - 1; x++) {
            double vn = (xr[x] * xr[x] - rxs * rxs) / m.sub_rad[x];
            for (int k = 0; k < m.sub_rad[x]; k++) {
                double r = std::sqrt(vn + ri * ri);
                m.radii.push_back(r);
                ri = r;
            }
            rxs = xr[x];
        }
        const double hpx = 0.5 * m.px, hpy = 0.5 * m.py;
        const double sep = TWOPI / m.sub_azi;
        for (int k = 0; k < m.sub_azi; k++) {
            Pt e = box_exit(Pt(-hpx, -hpy), Pt(hpx, hpy), Pt(0.0, 0.0), ang_from_at(k * sep, HPI, 0.0).alpha);
            m.lines.push_back(Seg{Pt(0.0, 0.0), e});
        }
        m.n_reg = ((int)m.radii.size() + 1) * m.sub_azi;
        double prev = 0.0;
        for (double r : m.radii) {
            double a = PI * (r * r - prev * prev) / m.sub_azi;
            for (int k = 0; k < m.sub_azi; k++) m.areas.push_back(a);
            prev = r;
        }
        double big = m.radii.back();
        double outer = (m.px * m.py - PI * big * big) / m.sub_azi;
        for (int k = 0; k < m.sub_azi; k++) m.areas.push_back(outer);
    } else if (t == "rect") {
        m.cyl = false;
        const Node *sx = n.child("sub_x"), *sy = n.child("sub_y");
        m.nx = sx ? std::atoi(sx->text.c_str()) : 0;
        m.ny = sy ? std::atoi(sy->text.c_str()) : 0;
        if (m.nx < 1 || m.ny < 1) throw Fail("Failed to read valid number of divisions in rect pin mesh.");
        m.n_xsreg = m.n_reg = m.nx * m.ny;
        const double dx = m.px / m.nx, dy = m.py / m.ny, hpx = 0.5 * m.px, hpy = 0.5 * m.py;
        for (int i = 0; i <= m.nx; i++) m.hx.push_back(i * dx - hpx);
        for (int i = 0; i <= m.ny; i++) m.hy.push_back(i * dy - hpy);
        for (size_t i = 1; i + 1 < m.hx.size(); i++) m.lines.push_back(Seg{Pt(m.hx[i], -hpy), Pt(m.hx[i], hpy)});
        for (size_t i = 1; i + 1 < m.hy.size(); i++) m.lines.push_back(Seg{Pt(-hpx, m.hy[i]), Pt(hpx, m.hy[i])});
        m.areas.assign(m.n_reg, dx * dy);
    } else {
        throw Fail("unsupported pin mesh type: " + t);
    }
    return m;
}

// ---- pins, lattices, core --------------------------------------------------------------
struct Pin {
    const PinMesh *mesh;
    vector<int> mats; // material ids per XS region
    bool fuel = false;
};
struct Lattice {
    int nx = 0, ny = 0;
    vector<const Pin *> pins; // row-major from the south row
    vector<double> xv, yv;    // pin boundaries
    vector<int> first_reg;    // per pin
    int n_reg = 0;
    const Pin &at(int ix, int iy) const { return *pins[(size_t)iy * nx + ix]; }
};

enum Surf { EAST = 0, NORTH = 1, WEST = 2, SOUTH = 3, TOP = 4, BOTTOM = 5, INVALID = 7 };

struct Core {
    int nlx = 0, nly = 0;              // lattices
    vector<const Lattice *> lats;      // row-major from the south row
    vector<double> lx, ly;             // lattice boundaries
    vector<int> lat_first_reg;
    vector<double> xv, yv, dx, dy;     // pin-cell boundaries and pitches
    int nx = 0, ny = 0, n_reg = 0, n_fuel = 0;
    double hx = 0, hy = 0, hz = 1.0;
    int bc[6];
    vector<Seg> lines;
    vector<const Pin *> pins;          // FSR order
    vector<int> pin_first_reg, pin_cell;

    // plane.cpp / lattice.cpp get_pinmesh with the default (+x, +y)
    // tie-break: the pin mesh at p, its first FSR, and p moved to the pin's
    // centre
    const PinMesh *pinmesh(Pt &p, int &first) const
    {
        unsigned ix = (unsigned)(std::lower_bound(lx.begin(), lx.end(), p.x, fuzzy_lt) - lx.begin());
        if (eq(p.x, lx[ix])) ix++;
        ix--;
        unsigned iy = (unsigned)(std::lower_bound(ly.begin(), ly.end(), p.y, fuzzy_lt) - ly.begin());
        if (eq(p.y, ly[iy])) iy++;
        iy--;
        ix = std::min((unsigned)nlx - 1, ix);
        iy = std::min((unsigned)nly - 1, iy);
        const size_t il = (size_t)nlx * iy + ix;
        const Lattice &L = *lats[il];
        first += lat_first_reg[il];
        Pt q(p.x - lx[ix], p.y - ly[iy]);
        unsigned jx = (unsigned)(std::lower_bound(L.xv.begin(), L.xv.end(), q.x, fuzzy_lt) - L.xv.begin());
        if (eq_abs(q.x, L.xv[jx])) jx++;
        jx--;
        jx = std::min((unsigned)L.nx - 1, jx);
        unsigned jy = (unsigned)(std::lower_bound(L.yv.begin(), L.yv.end(), q.y, fuzzy_lt) - L.yv.begin());
        if (eq_abs(q.y, L.yv[jy])) jy++;
        jy--;
        jy = std::min((unsigned)L.ny - 1, jy);
        q.x = 0.5 * (L.xv[jx + 1] + L.xv[jx]);
        q.y = 0.5 * (L.yv[jy + 1] + L.yv[jy]);
        first += L.first_reg[(size_t)jy * L.nx + jx];
        p = Pt(q.x + lx[ix], q.y + ly[iy]);
        return L.at(jx, jy).mesh;
    }
    int cell_of(Pt p) const
    {
        int ix = (int)(std::lower_bound(xv.begin(), xv.end(), p.x) - xv.begin()) - 1;
        int iy = (int)(std::lower_bound(yv.begin(), yv.end(), p.y) - yv.begin()) - 1;
        return iy * nx + ix;
    }
    // mesh.cpp prepare_surfaces
    int surf(int cell, int s) const
    {
        const int ix = cell % nx, iy = cell / nx;
        switch (s) {
        case EAST: return nx * ny + (nx + 1) * iy + ix + 1;
        case WEST: return nx * ny + (nx + 1) * iy + ix;
        case NORTH: return nx * ny + (nx + 1) * ny + (ny + 1) * ix + iy + 1;
        case SOUTH: return nx * ny + (nx + 1) * ny + (ny + 1) * ix + iy;
        case BOTTOM: return nx * iy + ix;
        default: return nx * ny + (nx + 1) * ny + (ny + 1) * nx + nx * iy + ix;
        }
    }
    int n_surf() const { return (nx + 1) * ny + (ny + 1) * nx + 2 * nx * ny; }
    // mesh.cpp Mesh::trace: crossings of the segment p1-p2 with the pin-cell
    // lines, sorted by y; crossings within 1e-10 cm of either end point (a
    // ray that starts or ends on a pin-cell corner) are not kept as pin
    // crossings of their own
    void trace(vector<Pt> &ps, bool literal) const
    {
        Seg l{ps[0], ps[1]};
        for (const Seg &li : lines) {
            Pt p;
            if (cross_lines(li, l, p) == 1) ps.push_back(p);
        }
        sort_unique(ps);
        if (!literal && ps.size() > 2) {
            const Pt a = ps.front(), b = ps.back();
            vector<Pt> kept{a};
            for (size_t k = 1; k + 1 < ps.size(); k++)
                if (!(std::hypot(ps[k].x - a.x, ps[k].y - a.y) < 1e-10 || std::hypot(ps[k].x - b.x, ps[k].y - b.y) < 1e-10))
                    kept.push_back(ps[k]);
            kept.push_back(b);
            ps.swap(kept);
        }
    }
    // mesh.cpp coarse_boundary_cell: the cell a ray enters the core through
    int boundary_cell(Pt p, int oct) const
    {
        bool on_x = false, on_y = false;
        int ix = 0;
        for (double xi : xv) {
            if (eq(p.x, xi)) {
                on_x = true;
                break;
            }
            if (xi > p.x) {
                ix--;
                break;
            }
            ix++;
        }
        int iy = 0;
        for (double yi : yv) {
            if (eq(p.y, yi)) {
                on_y = true;
                break;
            }
            if (yi > p.y) {
                iy--;
                break;
            }
            iy++;
        }
        if (eq_abs(p.x, 0.0)) {
            if (oct != 1 && on_y) iy--;
        } else if (eq(p.x, hx)) {
            ix--;
            if (oct != 2 && on_y) iy--;
        } else if (eq_abs(p.y, 0.0)) {
            if (oct != 1 && on_x) ix--;
        } else if (eq(p.y, hy)) {
            iy--;
            if (oct == 3 && on_x) ix--;
        }
        const int c = iy * nx + ix;
        if (ix < 0 || iy < 0 || ix >= nx || iy >= ny) throw Fail("ray starts outside the core");
        return c;
    }
    // mesh.cpp coarse_norm_point: the surface(s) a point on cell faces crosses
    int norm_point(Pt p, int oct, int (&s)[2]) const
    {
        bool on_x = false, on_y = false;
        int ix = 0;
        for (double xi : xv) {
            if (eq(p.x, xi)) {
                on_x = true;
                break;
            }
            if (xi > p.x) {
                ix--;
                break;
            }
            ix++;
        }
        int iy = 0;
        for (double yi : yv) {
            if (eq(p.y, yi)) {
                on_y = true;
                break;
            }
            if (yi > p.y) {
                iy--;
                break;
            }
            iy++;
        }
        if (!on_x && !on_y) return 0;
        if (on_x != on_y) {
            if (on_x) {
                if (ix == 0 && (oct == 1 || oct == 4)) return s[0] = WEST, 1;
                if (ix == nx && (oct == 2 || oct == 3)) return s[0] = EAST, 1;
            }
            if (on_y) {
                if (iy == 0 && (oct == 1 || oct == 2)) return s[0] = SOUTH, 1;
                if (iy == ny && (oct == 3 || oct == 4)) return s[0] = NORTH, 1;
            }
            if (on_x) s[0] = (oct == 1 || oct == 4) ? EAST : WEST;
            else s[0] = (oct == 1 || oct == 2) ? NORTH : SOUTH;
            return 1;
        }
        if (ix > 0 && ix < nx && iy > 0 && iy < ny) {
            s[0] = (oct == 1 || oct == 4) ? EAST : WEST;
            s[1] = (oct == 1 || oct == 2) ? NORTH : SOUTH;
            return 2;
        }
        if (ix == 0) {
            if (oct == 1 || oct == 4) return s[0] = WEST, 1;
            s[0] = (oct == 2) ? NORTH : SOUTH;
            s[1] = WEST;
            return 2;
        }
        if (ix == nx) {
            if (oct == 2 || oct == 3) return s[0] = EAST, 1;
            s[0] = (oct == 1) ? NORTH : SOUTH;
            s[1] = EAST;
            return 2;
        }
        if (iy == 0) {
            if (oct == 1 || oct == 2) return s[0] = SOUTH, 1;
            s[0] = (oct == 3) ? WEST : EAST;
            s[1] = SOUTH;
            return 2;
        }
        if (iy == ny) {
            if (oct == 3 || oct == 4) return s[0] = NORTH, 1;
            s[0] = (oct == 1) ? EAST : WEST;
            s[1] = NORTH;
            return 2;
        }
        return 0;
    }
};

struct Built {
    Library lib;
    vector<int> assigned;          // library index of each dense material
    std::map<int, int> id_dense;   // material id -> dense index
    std::map<int, PinMesh> meshes;
    std::map<int, Pin> pins;
    std::map<int, Lattice> lattices;
    Core core;
};

void build_core(const Node &doc, const string &xsl, Built &B)
{
    const Node *ml = doc.child("material_lib");
    if (!ml) throw Fail("No material library specified.");
    B.lib = read_xsl(xsl);
    for (const Node *m : ml->children("material")) {
        int id = m->integer("id", 0);
        auto it = B.lib.by_name.find(m->attr("name"));
        if (it == B.lib.by_name.end()) throw Fail("Failed to map material to ID: " + m->attr("name"));
        B.id_dense[id] = (int)B.assigned.size();
        B.assigned.push_back(it->second);
    }
    for (const Node *m : doc.children("mesh")) B.meshes[m->integer("id", 0)] = read_mesh(*m);
    for (const Node *p : doc.children("pin")) {
        Pin pin;
        auto mi = B.meshes.find(p->integer("mesh", 0));
        if (mi == B.meshes.end()) throw Fail("Invalid pin mesh ID.");
        pin.mesh = &mi->second;
        pin.mats = numbers<int>(p->text);
        if ((int)pin.mats.size() != pin.mesh->n_xsreg) throw Fail("Wrong number of materials specified in pin definition");
        for (int mid : pin.mats) {
            auto d = B.id_dense.find(mid);
            if (d == B.id_dense.end()) throw Fail("Invalid material specified in pin");
            if (B.lib.mats[B.assigned[d->second]].fissile) pin.fuel = true;
        }
        if (p->has("fuel")) pin.fuel = p->boolean("fuel", pin.fuel);
        B.pins[p->integer("id", 0)] = pin;
    }
    for (const Node *l : doc.children("lattice")) {
        Lattice L;
        L.nx = l->integer("nx", 0);
        L.ny = l->integer("ny", 0);
        vector<int> ids = numbers<int>(l->text);
        if ((int)ids.size() != L.nx * L.ny) throw Fail("Incorrect number of pin IDs specified for lattice.");
        L.pins.resize((size_t)L.nx * L.ny);
        // rows are listed from the north; stored from the south
        for (int iy = 0; iy < L.ny; iy++)
            for (int ix = 0; ix < L.nx; ix++) {
                auto pi = B.pins.find(ids[(size_t)iy * L.nx + ix]);
                if (pi == B.pins.end()) throw Fail("lattice names an unknown pin");
                L.pins[(size_t)(L.ny - iy - 1) * L.nx + ix] = &pi->second;
            }
        L.xv.push_back(0.0);
        for (int ix = 0; ix < L.nx; ix++) L.xv.push_back(L.xv.back() + L.at(ix, 0).mesh->px);
        L.yv.push_back(0.0);
        for (int iy = 0; iy < L.ny; iy++) L.yv.push_back(L.yv.back() + L.at(0, iy).mesh->py);
        int reg = 0;
        for (const Pin *p : L.pins) {
            L.first_reg.push_back(reg);
            reg += p->mesh->n_reg;
        }
        L.n_reg = reg;
        B.lattices[l->integer("id", 0)] = std::move(L);
    }
    std::map<int, const Lattice *> asy;
    std::map<int, double> asy_hz;
    for (const Node *a : doc.children("assembly")) {
        if (a->integer("np", 0) != 1) throw Fail("the oracle traces single-plane (2-D) assemblies only");
        const Node *ls = a->child("lattices");
        if (!ls) throw Fail("No lattices specified!");
        vector<int> ids = numbers<int>(ls->text);
        if (ids.size() != 1) throw Fail("Incorrect number of lattices specified for assembly.");
        auto li = B.lattices.find(ids[0]);
        if (li == B.lattices.end()) throw Fail("Unrecognized lattice ID in assembly.");
        asy[a->integer("id", 0)] = &li->second;
        asy_hz[a->integer("id", 0)] = a->dbl("hz", 1.0);
    }
    const Node *cn = nullptr;
    for (const Node *c : doc.children("core"))
        if (!c->has("enabled") || c->boolean("enabled", true)) {
            if (cn) throw Fail("More than one enabled core specification found.");
            cn = c;
        }
    if (!cn) throw Fail("No enabled core specifications.");
    Core &C = B.core;
    C.nlx = cn->integer("nx", 0);
    C.nly = cn->integer("ny", 0);
    const char *names[6] = {"east", "north", "west", "south", "top", "bottom"};
    for (int k = 0; k < 6; k++) {
        string v = cn->attr(names[k]);
        C.bc[k] = v == "vacuum" ? 0 : v == "reflect" ? 1 : v == "prescribed" ? 4 : -1;
        if (C.bc[k] < 0) throw Fail("Not all boundary conditions properly specified.");
    }
    vector<int> ids = numbers<int>(cn->text);
    if ((int)ids.size() != C.nlx * C.nly) throw Fail("Wrong number of assemblies specified for core.");
    C.lats.resize((size_t)C.nlx * C.nly);
    for (int iy = 0; iy < C.nly; iy++)
        for (int ix = 0; ix < C.nlx; ix++) {
            int id = ids[(size_t)iy * C.nlx + ix];
            if (!asy.count(id)) throw Fail("Failed to locate assembly in core specification.");
            C.lats[(size_t)(C.nly - iy - 1) * C.nlx + ix] = asy[id];
            C.hz = asy_hz[id];
        }
    C.lx.push_back(0.0);
    for (int ix = 0; ix < C.nlx; ix++) C.lx.push_back(C.lx.back() + C.lats[ix]->xv.back());
    C.ly.push_back(0.0);
    for (int iy = 0; iy < C.nly; iy++) C.ly.push_back(C.ly.back() + C.lats[(size_t)iy * C.nlx]->yv.back());
    C.hx = C.lx.back();
    C.hy = C.ly.back();
    int reg = 0;
    for (const Lattice *L : C.lats) {
        C.lat_first_reg.push_back(reg);
        reg += L->n_reg;
    }
    C.n_reg = reg;
    // pin-cell grid
    C.xv.push_back(0.0);
    for (int ix = 0; ix < C.nlx; ix++)
        for (int j = 0; j < C.lats[ix]->nx; j++) {
            double h = C.lats[ix]->at(j, 0).mesh->px;
            C.dx.push_back(h);
            C.xv.push_back(C.xv.back() + h);
        }
    C.yv.push_back(0.0);
    for (int iy = 0; iy < C.nly; iy++) {
        const Lattice &L = *C.lats[(size_t)iy * C.nlx];
        for (int j = 0; j < L.ny; j++) {
            double h = L.at(0, j).mesh->py;
            C.dy.push_back(h);
            C.yv.push_back(C.yv.back() + h);
        }
    }
    C.nx = (int)C.dx.size();
    C.ny = (int)C.dy.size();
    const double ext = std::max(C.hx, C.hy);
    for (size_t i = 1; i + 1 < C.xv.size(); i++) C.lines.push_back(Seg{Pt(C.xv[i], 0.0), Pt(C.xv[i], ext)});
    for (size_t i = 1; i + 1 < C.yv.size(); i++) C.lines.push_back(Seg{Pt(0.0, C.yv[i]), Pt(C.hx, C.yv[i])});
    // pins in FSR order: lattice by lattice, pin by pin; each pin's cell
    int r = 0, ox = 0, oy = 0;
    for (int ly = 0; ly < C.nly; ly++) {
        ox = 0;
        for (int lx = 0; lx < C.nlx; lx++) {
            const Lattice &L = *C.lats[(size_t)ly * C.nlx + lx];
            for (int jy = 0; jy < L.ny; jy++)
                for (int jx = 0; jx < L.nx; jx++) {
                    const Pin *p = &L.at(jx, jy);
                    C.pins.push_back(p);
                    C.pin_first_reg.push_back(r);
                    C.pin_cell.push_back((oy + jy) * C.nx + ox + jx);
                    r += p->mesh->n_reg;
                    if (p->fuel) C.n_fuel++;
                }
            ox += L.nx;
        }
        oy += C.lats[(size_t)ly * C.nlx]->ny;
    }
}

// ---- rays ---------------------------------------------------------------------------
std::pair<int, int> rational(double target, double tol)
{
    int a = 0, b = 1, c = 1, d = 1;
    const int max_d = std::numeric_limits<int>::max();
    if (std::fabs(double(a) / double(b) - target) < tol) return {a, b};
    if (std::fabs(double(c) / double(d) - target) < tol) return {c, d};
    while (b <= max_d && d <= max_d) {
        double m = double(a + c) / double(b + d);
        if (std::fabs(target - m) < tol) return {a + c, b + d};
        if (target > m) {
            a += c;
            b += d;
        } else {
            c += a;
            d += b;
        }
    }
    return {a, b};
}

struct Track {
    int bc0, bc1;
    vector<double> len;
    vector<int> reg;
    int cell_fw = 0, cell_bw = 0, surf_fw = 0, surf_bw = 0;
    vector<int> cm_fw, cm_bw, n_fw, n_bw;
};

struct Crossing {
    int cell, nseg;
    double len;
};

// Coarse walk of one direction: entry cell and surface, then every surface
// crossed with the segments before it (see the header for the rule)
void walk(const Core &C, const vector<Crossing> &px, int oct, Pt start, Pt end, int &cell0, int &surf0,
          vector<int> &surfs, vector<int> &nsegs)
{
    vector<int> cells, counts;
    int carry = 0;
    for (const Crossing &c : px) {
        if (c.len < 1e-9 && px.size() > 1) {
            if (counts.empty()) carry += c.nseg;
            else counts.back() += c.nseg;
            continue;
        }
        if (!cells.empty() && cells.back() == c.cell) {
            counts.back() += c.nseg + carry;
        } else {
            cells.push_back(c.cell);
            counts.push_back(c.nseg + carry);
        }
        carry = 0;
    }
    if (cells.empty()) throw Fail("ray crosses no pin");
    counts.back() += carry;
    int s[2];
    cell0 = cells.front();
    if (C.norm_point(start, oct, s) != 1) throw Fail("ray starts on more than one coarse surface");
    surf0 = C.surf(cell0, s[0]);
    for (size_t k = 0; k + 1 < cells.size(); k++) {
        const int dx = cells[k + 1] % C.nx - cells[k] % C.nx, dy = cells[k + 1] / C.nx - cells[k] / C.nx;
        const int fx = dx > 0 ? EAST : WEST, fy = dy > 0 ? NORTH : SOUTH;
        if (std::abs(dx) + std::abs(dy) == 1) {
            surfs.push_back(dx != 0 ? fx : fy);
            nsegs.push_back(counts[k]);
        } else if (std::abs(dx) == 1 && std::abs(dy) == 1) {
            surfs.push_back(fx);
            surfs.push_back(fy);
            nsegs.push_back(counts[k]);
            nsegs.push_back(0);
        } else {
            throw Fail("consecutive pin crossings are not neighbouring cells");
        }
    }
    const int ns = C.norm_point(end, oct, s);
    if (ns < 1) throw Fail("ray does not end on a coarse surface");
    for (int j = 0; j < ns; j++) surfs.push_back(s[j]);
    nsegs.push_back(counts.back());
    if (ns > 1) nsegs.push_back(0);
}

// MOCC's own coarse data of one direction (ray.cpp:84-145): the entry cell
// and surface from the start point, then the surface(s) of every pin-crossing
// end point by the fuzzy point test
void walk_literal(const Core &C, const vector<Pt> &cps, const vector<int> &nseg, int oct, int &cell0, int &surf0,
                  vector<int> &surfs, vector<int> &nsegs)
{
    int s[2];
    cell0 = C.boundary_cell(cps.front(), oct);
    if (C.norm_point(cps.front(), oct, s) != 1) throw Fail("ray starts on more than one coarse surface");
    surf0 = C.surf(cell0, s[0]);
    for (size_t k = 0; k < nseg.size(); k++) {
        const int ns = C.norm_point(cps[k + 1], oct, s);
        for (int j = 0; j < ns; j++) surfs.push_back(s[j]);
        nsegs.push_back(nseg[k]);
        if (ns > 1) nsegs.push_back(0);
    }
}

Track trace_ray(const Core &C, Pt p1, Pt p2, int bc0, int bc1, bool literal)
{
    Track T;
    T.bc0 = bc0;
    T.bc1 = bc1;
    vector<Pt> ps{p1, p2};
    C.trace(ps, literal);
    vector<Crossing> px;
    Pt prev = ps.front();
    for (size_t i = 1; i < ps.size(); i++) {
        Pt pc = mid(ps[i], prev);
        const Pt m = pc;
        int first = 0;
        const PinMesh *pm = C.pinmesh(pc, first);
        int n = pm->trace(Pt(prev.x - pc.x, prev.y - pc.y), Pt(ps[i].x - pc.x, ps[i].y - pc.y), first, T.len, T.reg);
        px.push_back(Crossing{C.cell_of(m), n, std::hypot(ps[i].x - prev.x, ps[i].y - prev.y)});
        prev = ps[i];
    }
    const int oct = (p2.x > p1.x) ? 1 : 2;
    vector<int> sf, sb, nf, nb;
    if (literal) {
        vector<int> ns;
        for (const Crossing &c : px) ns.push_back(c.nseg);
        walk_literal(C, ps, ns, oct, T.cell_fw, T.surf_fw, sf, nf);
        std::reverse(ps.begin(), ps.end());
        std::reverse(ns.begin(), ns.end());
        walk_literal(C, ps, ns, oct == 1 ? 3 : 4, T.cell_bw, T.surf_bw, sb, nb);
    } else {
        walk(C, px, oct, ps.front(), ps.back(), T.cell_fw, T.surf_fw, sf, nf);
        std::reverse(px.begin(), px.end());
        walk(C, px, oct == 1 ? 3 : 4, ps.back(), ps.front(), T.cell_bw, T.surf_bw, sb, nb);
    }
    const size_t n = std::min(nf.size(), nb.size());
    for (size_t i = 0; i < n; i++) {
        T.cm_fw.push_back(sf[i]);
        T.cm_bw.push_back(sb[i]);
        T.n_fw.push_back(nf[i]);
        T.n_bw.push_back(nb[i]);
    }
    if (nf.size() > nb.size()) {
        T.cm_fw.push_back(sf.back());
        T.cm_bw.push_back(INVALID);
        T.n_fw.push_back(0);
        T.n_bw.push_back(0);
    }
    if (nb.size() > nf.size()) {
        T.cm_fw.push_back(INVALID);
        T.cm_bw.push_back(sb.back());
        T.n_fw.push_back(0);
        T.n_bw.push_back(0);
    }
    return T;
}

} // namespace trc

// ---- the traced problem and its C interface ----------------------------------------
struct orc_traced {
    orc_problem p{};
    orc_options o{};
    std::map<std::string, std::vector<double>> d;
    std::map<std::string, std::vector<int>> i;
    std::vector<int64_t> seg_begin;
};

namespace trc {

void read_options(const Node &doc, orc_options &o, const Node *&sweeper)
{
    const Node *s = doc.child("solver");
    if (!s) throw Fail("No <solver> specified.");
    if (lower(s->attr("type")) != "eigenvalue") throw Fail("only <solver type=\"eigenvalue\"> is supported");
    o.k_tol = s->dbl("k_tol", -1.0);
    o.psi_tol = s->dbl("psi_tol", -1.0);
    o.max_iter = s->integer("max_iter", -1);
    if (o.k_tol <= 0.0 || o.psi_tol <= 0.0 || o.max_iter < 0) throw Fail("invalid eigenvalue solver tolerances");
    o.min_iter = s->has("min_iter") ? s->integer("min_iter", 0) : 0;
    o.cmfd = s->boolean("cmfd", false) ? 1 : 0;
    o.cmfd_enabled = 1;
    o.cmfd_k_tol = 1e-6;
    o.cmfd_psi_tol = 1e-5;
    o.cmfd_resid_reduction = 1e-3;
    o.cmfd_max_iter = 100;
    o.cmfd_negative_fixup = 0;
    if (const Node *c = s->child("cmfd")) {
        o.cmfd_k_tol = c->dbl("k_tol", o.cmfd_k_tol);
        o.cmfd_psi_tol = c->dbl("psi_tol", o.cmfd_psi_tol);
        o.cmfd_resid_reduction = c->dbl("residual_reduction", o.cmfd_resid_reduction);
        o.cmfd_max_iter = c->integer("max_iter", o.cmfd_max_iter);
        o.cmfd_negative_fixup = c->boolean("negative_fixup", false) ? 1 : 0;
        o.cmfd_enabled = c->boolean("enabled", true) ? 1 : 0;
    }
    sweeper = s->child("sweeper");
    if (!sweeper || lower(sweeper->attr("type")) != "moc") throw Fail("only <sweeper type=\"moc\"> is supported");
    o.n_inner = sweeper->integer("n_inner", -1);
    if (o.n_inner < 0) throw Fail("Invalid number of inner iterations specified (n_inner).");
    o.gs_boundary = 1;
    if (sweeper->has("boundary_update")) {
        std::string b = lower(sweeper->attr("boundary_update"));
        o.gs_boundary = (b == "jacobi" || b == "j") ? 0 : 1;
    }
    o.precision = 0;
    // not a MOCC attribute: enables MoCSweeper::update_incoming_flux, whose
    // call MOCC leaves commented out (eigen_solver.cpp:289)
    o.incoming_update = 0;
    if (sweeper->has("incoming_update")) {
        std::string u = lower(sweeper->attr("incoming_update"));
        if (u == "mocc") o.incoming_update = 1;
        else if (u == "surface") o.incoming_update = 2;
        else if (u != "off") throw Fail("Unrecognized incoming_update option (off|mocc|surface).");
    }
    // moc_sweeper.cpp:119: pugixml's as_bool, true when the value starts
    // with 1, t, T, y or Y
    o.tl_splitting = 0;
    if (sweeper->has("tl_splitting")) {
        const std::string v = sweeper->attr("tl_splitting");
        o.tl_splitting = (!v.empty() && std::string("1tTyY").find(v[0]) != std::string::npos) ? 1 : 0;
    }
}

Quad read_quad(const Node &q)
{
    Quad Q;
    std::string t = lower(q.attr("type"));
    Q.n_azi = q.integer("n_azimuthal", -1);
    Q.n_pol = q.integer("n_polar", -1);
    if (t == "ls" || t == "level-symmetric") {
        Q.type = LS;
        Q.ang = level_symmetric(q.integer("order", -1));
    } else if (t == "cg" || t == "chebyshev-gauss") {
        Q.type = CG;
        Q.ang = product(chebyshev(Q.n_azi), gauss(Q.n_pol));
    } else if (t == "cy" || t == "chebyshev-yamamoto") {
        Q.type = CY;
        Q.ang = product(chebyshev(Q.n_azi), yamamoto(Q.n_pol));
    } else {
        throw Fail("unsupported angular quadrature type: " + t);
    }
    Q.ndir = (int)Q.ang.size();
    Q.expand();
    return Q;
}

std::unique_ptr<orc_traced> trace_problem(const std::string &xml, const std::string &xsl, bool literal)
{
    auto doc = parse_xml(xml);
    auto out = std::make_unique<orc_traced>();
    const Node *sweeper = nullptr;
    read_options(*doc, out->o, sweeper);
    Built B;
    build_core(*doc, xsl, B);
    const Core &C = B.core;
    const Node *rn = sweeper->child("rays");
    if (!rn) throw Fail("No input privided for ray spacing.");
    const double spacing = rn->dbl("spacing", -1.0);
    if (spacing <= 0.0) throw Fail("Failed to read valid ray spacing.");
    // ray_data.cpp:67-134: volume correction, modularity, modularisation method
    const std::string corr = rn->has("volume_correction") ? lower(rn->attr("volume_correction")) : "flat";
    if (corr != "flat" && corr != "angle" && corr != "none")
        throw Fail("Unrecognized volume correction option in <rays>");
    bool core_modular = true;
    if (rn->has("modularity")) {
        const std::string mo = lower(rn->attr("modularity"));
        if (mo == "pin") core_modular = false;
        else if (mo != "core") throw Fail("Unrecognized modularity option.");
    }
    bool rational_mod = true;
    if (rn->has("modularization")) {
        const std::string mm = lower(rn->attr("modularization"));
        if (mm == "trig") rational_mod = false;
        else if (mm != "rational_fraction") throw Fail("Unrecognized modularization method specified.");
    }
    const Node *aq = sweeper->child("ang_quad");
    if (!aq && doc->child("solver")) aq = doc->child("solver")->child("ang_quad");
    if (!aq) aq = doc->child("ang_quad");
    if (!aq) throw Fail("No angular quadrature (<ang_quad>) found.");
    Quad Q = read_quad(*aq);

    // ray_data.cpp:136-206: modularise every octant-1 angle, over the core or
    // (pin modularity) over one pin cell, all of which must be alike
    double hx_mod = C.hx, hy_mod = C.hy;
    if (!core_modular) {
        hx_mod = C.pins.front()->mesh->px;
        hy_mod = C.pins.front()->mesh->py;
        for (const Pin *pn : C.pins)
            if (pn->mesh->px != hx_mod || pn->mesh->py != hy_mod)
                throw Fail("Core Mesh does not support pin modular ray tracing.");
    }
    const int nd = Q.ndir;
    std::vector<int> Nx1(nd), Ny1(nd);
    std::vector<double> sp1(nd);
    for (int ia = 0; ia < nd; ia++) {
        Ang a = Q.ang[ia];
        int Nx = 0, Ny = 0;
        if (rational_mod) {
            // RayData::modularize_angle, RATIONAL (ray_data.cpp:495-516)
            double m = (a.alpha < PI / 4.0) ? std::tan(a.alpha) : std::tan(PI / 2.0 - a.alpha);
            auto f = rational(m, 0.002);
            Nx = f.first;
            Ny = f.second;
            if (Nx == 0) throw Fail("azimuthal angle too shallow for rational modularisation");
            double al = std::atan((Nx * hy_mod) / (Ny * hx_mod));
            int scale = (int)std::ceil((hx_mod / Nx * std::fabs(std::sin(al))) / spacing);
            Nx *= scale;
            Ny *= scale;
            if (a.alpha > PI / 4.0) std::swap(Nx, Ny);
        } else {
            // TRIG (ray_data.cpp:517-523): ray counts from the nominal
            // spacing, rounded up to even
            Nx = (int)std::ceil(hx_mod / spacing * std::fabs(std::sin(a.alpha)));
            Ny = (int)std::ceil(hy_mod / spacing * std::fabs(std::cos(a.alpha)));
            Nx += Nx % 2;
            Ny += Ny % 2;
        }
        if (!core_modular) {
            Nx *= C.nx;
            Ny *= C.ny;
        }
        Ang b = ang_from_at(std::atan(C.hy * Nx / (C.hx * Ny)), a.theta, a.w);
        Q.modify(ia, b);
        Nx1[ia] = Nx;
        Ny1[ia] = Ny;
        sp1[ia] = std::cos(Q.ang[ia].alpha) * C.hy / Ny;
    }
    Q.update_weights();
    const int pps = (Q.type == LS) ? 1 : Q.n_pol;
    const int sets_oct = nd / pps;
    const int n_sets = 2 * sets_oct;

    // trace one set of tracks per azimuth in octants 1 and 2
    std::vector<std::vector<Track>> sets(n_sets);
    std::vector<int> snx(n_sets), sny(n_sets);
    std::vector<double> ssp(n_sets);
    const Pt lo(0.0, 0.0), hi(C.hx, C.hy);
    for (int s = 0; s < n_sets; s++) {
        const int ia = (s / sets_oct) * nd + (s % sets_oct) * pps;
        const Ang &a = Q.ang[ia];
        const int Nx = Nx1[ia % nd], Ny = Ny1[ia % nd];
        const double sp = sp1[ia % nd];
        snx[s] = Nx;
        sny[s] = Ny;
        ssp[s] = sp;
        const double spx = std::fabs(sp / std::sin(a.alpha)), spy = std::fabs(sp / std::cos(a.alpha));
        auto exit_bc = [&](const Pt &p2) -> int {
            if (eq(p2.x, C.hx)) return (int)(p2.y / spy);
            if (eq(p2.y, C.hy)) return (int)(p2.x / spx) + Ny;
            if (eq(p2.x, 0.0)) return (int)(p2.y / spy);
            throw Fail("Something has gone horribly wrong in the ray trace.");
        };
        for (int k = 0; k < Ny; k++) {
            Pt p1((a.ox > 0.0) ? 0.0 : C.hx, (0.5 + k) * spy);
            Pt p2 = box_exit(lo, hi, p1, a.alpha);
            sets[s].push_back(trace_ray(C, p1, p2, k, exit_bc(p2), literal));
        }
        for (int k = 0; k < Nx; k++) {
            Pt p1((0.5 + k) * spx, 0.0);
            Pt p2 = box_exit(lo, hi, p1, a.alpha);
            sets[s].push_back(trace_ray(C, p1, p2, k + Ny, exit_bc(p2), literal));
        }
    }
    std::vector<double> area;
    for (const Pin *p : C.pins) area.insert(area.end(), p->mesh->areas.begin(), p->mesh->areas.end());
    if (corr == "flat") {
        // ray_data.cpp:348-411: each angle's lengths scaled so that its
        // segments' volumes equal every FSR's area (the polar angles of a
        // set share its tracks and get the same factor)
        for (int s = 0; s < n_sets; s++) {
            std::vector<double> vol(C.n_reg, 0.0);
            for (const Track &t : sets[s])
                for (size_t k = 0; k < t.len.size(); k++) vol[t.reg[k]] += t.len[k] * ssp[s];
            std::vector<double> cf(C.n_reg);
            for (int r = 0; r < C.n_reg; r++) cf[r] = area[r] / vol[r];
            for (Track &t : sets[s])
                for (size_t k = 0; k < t.len.size(); k++) t.len[k] = t.len[k] * cf[t.reg[k]];
        }
    } else if (corr == "angle") {
        // ray_data.cpp:414-474: one factor per FSR from the weighted volume
        // integral over every angle of octants 1 and 2 (weight / 2 each),
        // applied to every angle's lengths
        std::vector<double> vol(C.n_reg, 0.0);
        for (int s = 0; s < n_sets; s++) {
            const int ia0 = (s / sets_oct) * nd + (s % sets_oct) * pps;
            for (int p = 0; p < pps; p++) {
                const double wgt = Q.ang[ia0 + p].w * 0.5;
                for (const Track &t : sets[s])
                    for (size_t k = 0; k < t.len.size(); k++) vol[t.reg[k]] += t.len[k] * ssp[s] * wgt;
            }
        }
        for (int r = 0; r < C.n_reg; r++) vol[r] = area[r] / vol[r];
        for (int s = 0; s < n_sets; s++)
            for (Track &t : sets[s])
                for (size_t k = 0; k < t.len.size(); k++) t.len[k] = t.len[k] * vol[t.reg[k]];
    }

    // ---- flatten ----
    auto &D = out->d;
    auto &I = out->i;
    const int G = B.lib.ng;
    for (int li : B.assigned) {
        const Material &m = B.lib.mats[li];
        D["xstr"].insert(D["xstr"].end(), m.xstr.begin(), m.xstr.end());
        D["xsnf"].insert(D["xsnf"].end(), m.xsnf.begin(), m.xsnf.end());
        D["xsf"].insert(D["xsf"].end(), m.xsf.begin(), m.xsf.end());
        D["xsch"].insert(D["xsch"].end(), m.xsch.begin(), m.xsch.end());
        D["scat"].insert(D["scat"].end(), m.scat.begin(), m.scat.end());
    }
    for (const Pin *p : C.pins)
        for (size_t x = 0; x < p->mats.size(); x++)
            for (int k = 0; k < p->mesh->fsrs_of((int)x); k++) I["fsr_mat"].push_back(B.id_dense.at(p->mats[x]));
    D["fsr_area"] = area;
    for (double a : area) D["fsr_vol"].push_back(a * C.hz);
    for (int ia = 0; ia < 4 * nd; ia++) {
        const Ang &a = Q.ang[ia];
        D["ang_ox"].push_back(a.ox);
        D["ang_oy"].push_back(a.oy);
        D["ang_oz"].push_back(a.oz);
        D["ang_alpha"].push_back(a.alpha);
        D["ang_theta"].push_back(a.theta);
        D["ang_weight"].push_back(a.w);
        D["ang_rsintheta"].push_back(a.rsin);
    }
    // every angle of the (modularised) quadrature, 8 octants, and the group
    // bounds: what AngularQuadrature::output and FixedSourceSolver::output
    // write (angular_quadrature.cpp:213-248, fixed_source_solver.cpp:119-129)
    for (const Ang &a : Q.ang) {
        D["quad_alpha"].push_back(a.alpha);
        D["quad_theta"].push_back(a.theta);
        D["quad_ox"].push_back(a.ox);
        D["quad_oy"].push_back(a.oy);
        D["quad_oz"].push_back(a.oz);
        D["quad_weight"].push_back(a.w);
    }
    I["quad_n"] = {Q.n_pol, Q.n_azi};
    D["group_bounds"] = B.lib.bounds;
    I["set_nx"] = snx;
    I["set_ny"] = sny;
    D["set_spacing"] = ssp;
    out->seg_begin.push_back(0);
    I["trk_cm_begin"].push_back(0);
    int n_tracks = 0;
    for (int s = 0; s < n_sets; s++) {
        I["set_first_track"].push_back(n_tracks);
        for (const Track &t : sets[s]) {
            I["trk_bc0"].push_back(t.bc0);
            I["trk_bc1"].push_back(t.bc1);
            I["trk_set"].push_back(s);
            D["seg_len"].insert(D["seg_len"].end(), t.len.begin(), t.len.end());
            I["seg_fsr"].insert(I["seg_fsr"].end(), t.reg.begin(), t.reg.end());
            out->seg_begin.push_back((int64_t)D["seg_len"].size());
            I["trk_cm_cell_fw"].push_back(t.cell_fw);
            I["trk_cm_cell_bw"].push_back(t.cell_bw);
            I["trk_cm_surf_fw"].push_back(t.surf_fw);
            I["trk_cm_surf_bw"].push_back(t.surf_bw);
            I["cm_fw"].insert(I["cm_fw"].end(), t.cm_fw.begin(), t.cm_fw.end());
            I["cm_bw"].insert(I["cm_bw"].end(), t.cm_bw.begin(), t.cm_bw.end());
            I["cm_nseg_fw"].insert(I["cm_nseg_fw"].end(), t.n_fw.begin(), t.n_fw.end());
            I["cm_nseg_bw"].insert(I["cm_nseg_bw"].end(), t.n_bw.begin(), t.n_bw.end());
            I["trk_cm_begin"].push_back((int)I["cm_fw"].size());
            n_tracks++;
        }
    }
    I["set_first_track"].push_back(n_tracks);
    D["dx"] = C.dx;
    D["dy"] = C.dy;
    I["pin_first_reg"] = C.pin_first_reg;
    I["pin_first_reg"].push_back(C.n_reg);
    I["pin_cell"] = C.pin_cell;
    for (const Pin *p : C.pins) {
        I["pin_fuel"].push_back(p->fuel ? 1 : 0);
        D["pin_area"].push_back(p->mesh->px * p->mesh->py);
    }
    // make every named array exist, even when empty
    for (const char *k : {"cm_fw", "cm_bw", "cm_nseg_fw", "cm_nseg_bw", "seg_fsr"}) I[k];
    D["seg_len"];

    orc_problem &p = out->p;
    p.ng = G;
    p.n_fsr = C.n_reg;
    p.n_mat = (int)B.assigned.size();
    p.ndir_oct = nd;
    p.n_ang = 4 * nd;
    p.n_sets = n_sets;
    p.pol_per_set = pps;
    p.nx = C.nx;
    p.ny = C.ny;
    p.n_pin = C.nx * C.ny;
    p.n_surf = C.n_surf();
    p.n_fuel_2d = C.n_fuel;
    p.n_tracks = n_tracks;
    p.n_seg = (int64_t)D["seg_len"].size();
    p.hz = C.hz;
    for (int k = 0; k < 6; k++) p.bc[k] = C.bc[k];
    p.xstr = D["xstr"].data();
    p.xsnf = D["xsnf"].data();
    p.xsf = D["xsf"].data();
    p.xsch = D["xsch"].data();
    p.scat = D["scat"].data();
    p.fsr_mat = I["fsr_mat"].data();
    p.fsr_vol = D["fsr_vol"].data();
    p.fsr_area = D["fsr_area"].data();
    p.ang_ox = D["ang_ox"].data();
    p.ang_oy = D["ang_oy"].data();
    p.ang_oz = D["ang_oz"].data();
    p.ang_alpha = D["ang_alpha"].data();
    p.ang_theta = D["ang_theta"].data();
    p.ang_weight = D["ang_weight"].data();
    p.ang_rsintheta = D["ang_rsintheta"].data();
    p.set_nx = I["set_nx"].data();
    p.set_ny = I["set_ny"].data();
    p.set_first_track = I["set_first_track"].data();
    p.set_spacing = D["set_spacing"].data();
    p.trk_bc0 = I["trk_bc0"].data();
    p.trk_bc1 = I["trk_bc1"].data();
    p.trk_set = I["trk_set"].data();
    p.trk_seg_begin = out->seg_begin.data();
    p.trk_cm_cell_fw = I["trk_cm_cell_fw"].data();
    p.trk_cm_cell_bw = I["trk_cm_cell_bw"].data();
    p.trk_cm_surf_fw = I["trk_cm_surf_fw"].data();
    p.trk_cm_surf_bw = I["trk_cm_surf_bw"].data();
    p.trk_cm_begin = I["trk_cm_begin"].data();
    p.cm_fw = I["cm_fw"].data();
    p.cm_bw = I["cm_bw"].data();
    p.cm_nseg_fw = I["cm_nseg_fw"].data();
    p.cm_nseg_bw = I["cm_nseg_bw"].data();
    p.seg_len = D["seg_len"].data();
    p.seg_fsr = I["seg_fsr"].data();
    p.dx = D["dx"].data();
    p.dy = D["dy"].data();
    p.pin_first_reg = I["pin_first_reg"].data();
    p.pin_cell = I["pin_cell"].data();
    p.pin_fuel = I["pin_fuel"].data();
    p.pin_area = D["pin_area"].data();
    return out;
}

} // namespace trc

static thread_local std::string g_trace_error;

extern "C" {

const char *orc_trace_error(void) { return g_trace_error.c_str(); }

int orc_trace(const char *xml, const char *xsl, int mocc_literal, orc_traced **out)
{
    try {
        if (!xml || !xsl || !out) throw trc::Fail("null argument");
        *out = trc::trace_problem(xml, xsl, mocc_literal != 0).release();
        return 0;
    } catch (const std::exception &e) {
        g_trace_error = e.what();
        return 1;
    }
}

void orc_traced_destroy(orc_traced *t) { delete t; }

const orc_problem *orc_traced_problem(const orc_traced *t) { return &t->p; }
const orc_options *orc_traced_options(const orc_traced *t) { return &t->o; }

/* one named array of the traced problem: *kind 0 int32, 1 double, 2 int64 */
int orc_traced_array(const orc_traced *t, const char *name, const void **data, int64_t *n, int *kind)
{
    std::string k(name);
    if (k == "trk_seg_begin") {
        *data = t->seg_begin.data();
        *n = (int64_t)t->seg_begin.size();
        *kind = 2;
        return 0;
    }
    auto di = t->d.find(k);
    if (di != t->d.end()) {
        *data = di->second.data();
        *n = (int64_t)di->second.size();
        *kind = 1;
        return 0;
    }
    auto ii = t->i.find(k);
    if (ii != t->i.end()) {
        *data = ii->second.data();
        *n = (int64_t)ii->second.size();
        *kind = 0;
        return 0;
    }
    g_trace_error = "no traced array named " + k;
    return 1;
}
}
