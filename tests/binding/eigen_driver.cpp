// MOCC's EigenSolver::solve / step (src/solvers/eigen_solver.cpp:131-253) and
// FixedSourceSolver::step (src/solvers/fixed_source_solver.cpp:102-117)
// driving the GPU sweeper through the TransportSweeper interface only, as a
// MOCC build with MoCSweeperGPU would. Usage:
//   eigen_driver input.xml [library.xsl|-] [precision]
// prints {"k", "iterations", "converged", "error_k", "error_psi"} as JSON;
// exit status 2 on a MOCC exception, 3 when the library reports no GPU.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

#include "moc_sweeper_gpu.hpp"

using mocc::ArrayB1;
using mocc::real_t;

static std::string slurp(const std::string &path)
{
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot read " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// Normalize (src/util/utils.hpp:29-51): scale to a mean of one over the
// positive entries
static void normalize(ArrayB1 &v)
{
    int n = 0;
    double sum = 0.0;
    for (real_t x : v.v) {
        if (x > 0.0) n++;
        sum += x;
    }
    const double f = (double)n / sum;
    for (real_t &x : v.v) x *= f;
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s input.xml [library.xsl|-] [precision]\n", argv[0]);
        return 1;
    }
    const std::string xml_path = argv[1];
    const std::string xsl = (argc > 2 && std::string(argv[2]) != "-") ? slurp(argv[2]) : std::string();
    const int precision = argc > 3 ? std::atoi(argv[3]) : -1;
    const std::string base = xml_path.find('/') == std::string::npos ? "." : xml_path.substr(0, xml_path.rfind('/'));
    try {
        mocc::moc::MoCSweeperGPU S(slurp(xml_path), xsl, base, precision);
        const mocgpu_options &o = S.options();
        mocc::CoarseData cd;
        const bool cmfd = o.cmfd && o.cmfd_enabled;
        if (cmfd) S.set_coarse_data(&cd);
        S.initialize();

        real_t k = 1.0, k_prev = 1.0, error_k = o.k_tol, error_psi = o.psi_tol;
        ArrayB1 fs(S.n_reg()), fs_prev(S.n_reg());
        S.calc_fission_source(k, fs);
        int n_fissile = 0;
        for (real_t x : fs.v) n_fissile += x > 0.0 ? 1 : 0;
        int it = 0, converged = 0;
        for (; it < o.max_iter; it++) {
            // EigenSolver::step
            if (cmfd) S.cmfd(k); // do_cmfd
            S.calc_fission_source(k, fs);
            fs_prev = fs;
            // FixedSourceSolver::step
            S.store_old_flux();
            for (int g = 0; g < S.n_group(); g++) {
                S.build_source(g);
                S.sweep(g);
            }
            const real_t tfis1 = S.total_fission(false), tfis2 = S.total_fission(true);
            k_prev = k;
            k = k * tfis1 / tfis2;
            S.calc_fission_source(k, fs);
            // EigenSolver::solve's convergence test
            error_k = std::fabs(k - k_prev);
            ArrayB1 a = fs, b = fs_prev;
            normalize(a);
            normalize(b);
            double efis = 0.0;
            for (int i = 0; i < S.n_reg(); i++) efis += (a(i) - b(i)) * (a(i) - b(i));
            error_psi = std::sqrt(efis / n_fissile);
            if (k != k) throw mocc::Exception(__FILE__, __LINE__, __func__, "Eigenvalue is not a number. Giving up.");
            if (error_k < o.k_tol && error_psi < o.psi_tol && it >= o.min_iter) {
                converged = 1;
                it++;
                break;
            }
        }
        std::printf("{\"k\": %.17g, \"iterations\": %d, \"converged\": %d, \"error_k\": %.6g, \"error_psi\": %.6g}\n", k,
                    it, converged, error_k, error_psi);
    } catch (const mocc::Exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return std::string(e.what()).find("CUDA") != std::string::npos ? 3 : 2;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 2;
    }
    return 0;
}
