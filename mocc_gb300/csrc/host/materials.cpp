#include "materials.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <regex>
#include <sstream>

#include "geom.hpp"
#include "xml.hpp"

namespace mocgpu {

void Material::finalize()
{
    fissile = std::any_of(xsnf.begin(), xsnf.end(), [](double v) { return v > 0.0; });
    if (std::any_of(xsch.begin(), xsch.end(), [](double v) { return v > 0.0; })) {
        double sum = 0.0;
        for (double c : xsch) sum += c;
        for (double &c : xsch) c /= sum;
    }
    // Out-scatter sums each "from" column over the band of every "to" row
    // (the band spans the positive entries, so it equals the column sum).
    out.assign(ng, 0.0);
    for (int to = 0; to < ng; to++) {
        int lo = to, hi = to;
        for (int f = 0; f < ng; f++)
            if (s(to, f) > 0.0) { lo = std::min(f, to); break; }
        for (int f = ng - 1; f >= 0; f--)
            if (s(to, f) > 0.0) { hi = std::max(f, to); break; }
        for (int f = lo; f <= hi; f++) out[f] += s(to, f);
    }
    xstr.resize(ng);
    for (int g = 0; g < ng; g++) xstr[g] = xsab[g] + out[g];
}

namespace {
std::string trim(const std::string &s)
{
    size_t b = s.find_first_not_of(" \t\r\n");
    if (b == std::string::npos) return "";
    size_t e = s.find_last_not_of(" \t\r\n");
    return s.substr(b, e - b + 1);
}

struct Scrubber {
    std::istringstream in;
    explicit Scrubber(const std::string &t) : in(t) {}
    std::string getline()
    {
        std::string line;
        while (std::getline(in, line)) {
            size_t c = line.find('!');
            if (c != std::string::npos) line.erase(c);
            line = trim(line);
            if (!line.empty()) return line;
        }
        return "";
    }
};
} // namespace

MaterialLib MaterialLib::from_xsl_text(const std::string &text)
{
    MaterialLib ml;
    Scrubber sc(text);
    sc.getline(); // description
    int nmat = 0;
    {
        std::istringstream b(sc.getline());
        b >> ml.ng >> nmat;
        if (b.fail() || ml.ng <= 0 || nmat <= 0) MOCGPU_THROW(4, "bad .xsl header");
    }
    {
        std::istringstream b(sc.getline());
        for (int g = 0; g < ml.ng; g++) {
            double v;
            b >> v;
            if (b.fail()) MOCGPU_THROW(4, "trouble reading group bounds");
            ml.group_bounds.push_back(v);
        }
    }
    std::regex head("^\\s*XSMACRO\\s+([^\\s]+)\\s+([0-9]+)\\s*$");
    for (int m = 0; m < nmat; m++) {
        std::string line = sc.getline();
        std::smatch res;
        if (!std::regex_match(line, res, head)) MOCGPU_THROW(4, "bad XSMACRO header: " + line);
        Material mat;
        mat.name = res[1].str();
        mat.ng = ml.ng;
        mat.xsab.resize(ml.ng);
        mat.xsnf.resize(ml.ng);
        mat.xsf.resize(ml.ng);
        mat.xsch.resize(ml.ng);
        for (int g = 0; g < ml.ng; g++) {
            auto v = explode<double>(sc.getline());
            if (v.size() != 4) MOCGPU_THROW(4, "trouble reading XS data from library");
            mat.xsab[g] = v[0];
            mat.xsnf[g] = v[1];
            mat.xsf[g] = v[2];
            mat.xsch[g] = v[3];
        }
        mat.scat.assign((size_t)ml.ng * ml.ng, 0.0);
        for (int to = 0; to < ml.ng; to++) {
            auto v = explode<double>(sc.getline());
            if ((int)v.size() != ml.ng) MOCGPU_THROW(4, "trouble reading scattering row");
            for (int f = 0; f < ml.ng; f++) mat.scat[(size_t)to * ml.ng + f] = v[f];
        }
        mat.finalize();
        // a solve on a non-finite or non-positive transport cross section
        // would only end in a NaN eigenvalue: refuse the library instead
        for (int g = 0; g < ml.ng; g++) {
            const double vals[5] = {mat.xstr[g], mat.xsab[g], mat.xsnf[g], mat.xsf[g], mat.xsch[g]};
            for (double v : vals)
                if (!std::isfinite(v)) MOCGPU_THROW(4, "non-finite cross section in material " + mat.name);
            if (!(mat.xstr[g] > 0.0))
                MOCGPU_THROW(4, "non-positive transport cross section in material " + mat.name + ", group " +
                                    std::to_string(g + 1));
        }
        for (double v : mat.scat)
            if (!std::isfinite(v)) MOCGPU_THROW(4, "non-finite scattering cross section in material " + mat.name);
        ml.by_name[mat.name] = m;
        ml.lib.push_back(std::move(mat));
    }
    return ml;
}

void MaterialLib::assign(int id, const std::string &name)
{
    auto it = by_name.find(name);
    if (it == by_name.end()) MOCGPU_THROW(4, "material not in library: " + name);
    id_to_dense[id] = (int)assigned.size();
    assigned.push_back(lib[it->second]);
}

const Material &MaterialLib::by_id(int id) const
{
    auto it = id_to_dense.find(id);
    if (it == id_to_dense.end()) MOCGPU_THROW(4, "invalid material id " + std::to_string(id));
    return assigned[it->second];
}

// ---------------------------------------------------------------------------
// Synthetic library. Raw 64-bit draws come from a splitmix64 stream so that
// the library is bit-identical on every host.
namespace {
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double a, double b) { return a + (b - a) * uniform(); }
    double log_uniform(double a, double b) { return std::exp(uniform(std::log(a), std::log(b))); }
};

Material make_material(Rng &rng, const std::string &name, int ng, bool fuel)
{
    Material m;
    m.name = name;
    m.ng = ng;
    m.xsab.assign(ng, 0.0);
    m.xsnf.assign(ng, 0.0);
    m.xsf.assign(ng, 0.0);
    m.xsch.assign(ng, 0.0);
    m.scat.assign((size_t)ng * ng, 0.0);
    const int n_chi = std::max(3, (int)std::lround(3.0 * ng / 7.0));
    const int n_up = std::max(2, (int)std::lround(2.0 * ng / 7.0)); // upscatter targets
    const double nu = 2.43;
    for (int f = 0; f < ng; f++) {
        double st = rng.log_uniform(0.2, 2.0);
        double c = rng.uniform(0.4, 0.95);
        // Split the out-scatter of group f: self-scatter, downscatter into the
        // next two groups, and (for the last groups only) a small upscatter.
        std::vector<double> w(ng, 0.0);
        w[f] = rng.uniform(0.4, 0.8);
        for (int k = 1; k <= 2 && f + k < ng; k++) w[f + k] = rng.uniform(0.05, 0.4) / k;
        if (f > 0 && f - 1 >= ng - n_up) w[f - 1] = rng.uniform(0.01, 0.05);
        double wsum = 0.0;
        for (double v : w) wsum += v;
        for (int to = 0; to < ng; to++) m.scat[(size_t)to * ng + f] = c * st * w[to] / wsum;
        m.xsab[f] = st * (1.0 - c);
        if (fuel) {
            m.xsnf[f] = rng.uniform(0.005, 0.5);
            m.xsf[f] = m.xsnf[f] / nu;
            if (f < n_chi) m.xsch[f] = rng.uniform(0.1, 1.0);
        }
    }
    return m;
}
} // namespace

std::string synthetic_xsl(const SyntheticXsSpec &spec)
{
    if (spec.ng < 3) MOCGPU_THROW(1, "synthetic library needs at least 3 groups");
    Rng rng(spec.seed);
    std::vector<Material> mats;
    Material base_fuel = make_material(rng, "fuel", spec.ng, true);
    for (int i = 0; i < spec.n_fuel; i++) {
        Material f = base_fuel;
        f.name = "fuel" + std::to_string(i + 1);
        double sc = (i < (int)spec.fuel_nf_scale.size()) ? spec.fuel_nf_scale[i] : 1.0;
        for (int g = 0; g < spec.ng; g++) {
            f.xsnf[g] *= sc * spec.fuel_nf_factor;
            f.xsf[g] *= sc * spec.fuel_nf_factor;
        }
        mats.push_back(f);
    }
    Material mod = make_material(rng, "moderator", spec.ng, false);
    for (int g = 0; g < spec.ng; g++) mod.xsab[g] *= spec.mod_factor;
    for (double &v : mod.scat) v *= spec.mod_factor;
    mats.push_back(mod);

    std::string out;
    char buf[64];
    out += "Synthetic macroscopic cross sections\n";
    out += " " + std::to_string(spec.ng) + " " + std::to_string(mats.size()) + "\n";
    for (int g = 0; g < spec.ng; g++) {
        std::snprintf(buf, sizeof(buf), " %.6e", 2.0e7 * std::pow(1.0e-8, (double)g / spec.ng));
        out += buf;
    }
    out += "\n";
    for (const auto &m : mats) {
        out += "XSMACRO " + m.name + " 0\n";
        for (int g = 0; g < spec.ng; g++) {
            std::snprintf(buf, sizeof(buf), " %.17e", m.xsab[g]);
            out += buf;
            std::snprintf(buf, sizeof(buf), " %.17e", m.xsnf[g]);
            out += buf;
            std::snprintf(buf, sizeof(buf), " %.17e", m.xsf[g]);
            out += buf;
            std::snprintf(buf, sizeof(buf), " %.17e\n", m.xsch[g]);
            out += buf;
        }
        for (int to = 0; to < spec.ng; to++) {
            for (int f = 0; f < spec.ng; f++) {
                std::snprintf(buf, sizeof(buf), " %.17e", m.s(to, f));
                out += buf;
            }
            out += "\n";
        }
    }
    return out;
}

} // namespace mocgpu
