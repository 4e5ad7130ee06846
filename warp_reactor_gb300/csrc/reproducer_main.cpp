// reproducer_main.cpp -- the drop-in reproducer program for the GB300 library.
//
// Same command line, standard output, output files and exit codes as the
// reference program's CUDA build (reproducer.cpp:7978-8702), with the grid
// integration done by libwarp_reactor through the C ABI:
//
//   --grid N                      grid dimension (N^3 cells), default 64
//   --perturb | --no-perturb      seeded density perturbations (default on)
//   --compare-final-state FILE    compare with a final_states_grid<N> file
//   --compare-final-state=FILE
//   --no-compare-final-state      (default for the GPU backend)
//   --math cuda|portable          exp/log arithmetic (this program only;
//                                 default cuda: CUDA's libm, the arithmetic of
//                                 the reference's CUDA build; see warp_reactor.h)
//   --driver-policy gridwide-independent|legacy-local|gridwide-cta32
//                                 outer-step policy (default gridwide-independent;
//                                 legacy-local is the reference CPU program's,
//                                 gridwide-cta32 its structured CUDA build's)
//   --write-final-state FILE      also write the packed final states to FILE with
//                                 a FILE.manifest sidecar; refuses to overwrite
//                                 either (the reference's Mojo program's flag,
//                                 reproducer.mojo:3283-3330)
//   -h | --help
//
// Output files: final_states_grid<N>_cuda.bin (grid > 1), rotated to
// <file>.old.NNNNNN when it exists; final_state_comparison_failures_cuda.csv on a
// failed comparison.  The backend name "cuda" is the reference CUDA program's, so
// scripts written for it find the same files.
#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <string_view>
#include <vector>

#include "warp_reactor.h"

namespace {

constexpr int kDefaultGrid = 64;
constexpr double kAtolSpec = 1.0e-4;          // reproducer.cpp:7411
constexpr double kAtolEnergy = 1.0e-6;        // :7413
constexpr double kRtolSpec = 1.0e-4;          // :7410
constexpr double kThermoRtol = 2.0e-4;        // :7414
constexpr int kBackupDigits = 6;              // :7420-7422
constexpr int kBackupLimit = 1000000;
constexpr int kBackupAttempts = 100;
// comparison_species_rtol, reproducer.cpp:7429-7431
constexpr double kSpeciesRtol[WR_NUM_SPECIES] = {1.0e-3, 1.0e-3, 1.1e-3, 1.0e-3, 1.0e-4, 10.0, 1.0e-3,
                                                 1.0e-4, 3.0e-4, 1.0e-4, 10.0, 1.0e-4, 1.0e-4, 1.0e-4};
constexpr const char* kSpecNames[WR_NUM_SPECIES] = {"E",  "Hp", "H",  "Hm",  "Dp",   "D",   "H2p",
                                                    "Dm", "H2", "HDp", "HD", "HEpp", "HEp", "HE"};
constexpr const char* kBackend = "cuda";

struct Options {
    int grid_dim = kDefaultGrid;
    bool perturb = true;
    bool show_help = false;
    int math = WR_MATH_CUDA;
    int policy = WR_POLICY_GRIDWIDE_INDEPENDENT;
    std::string write_path;
    std::string compare_path;  // the GPU backend compares only on request (:7467-7468)
};

bool is_deuterium_bearing(int n) { return n == 4 || n == 5 || n == 7 || n == 9 || n == 10; }

struct CounterSummary {
    uint64_t min{};
    long double median{};
    uint64_t max{};
};
struct ValueSummary {
    long double min{}, median{}, max{};
};

// summarize_counter / summarize_value, reproducer.cpp:7988-8024
CounterSummary summarize_counter(std::vector<uint64_t> v) {
    std::sort(v.begin(), v.end());
    const size_t n = v.size();
    const long double med = (n % 2 == 1) ? static_cast<long double>(v[n / 2])
                                         : (static_cast<long double>(v[n / 2 - 1]) + static_cast<long double>(v[n / 2])) / 2.0L;
    return {v.front(), med, v.back()};
}
ValueSummary summarize_value(std::vector<long double> v) {
    std::sort(v.begin(), v.end());
    const size_t n = v.size();
    const long double med = (n % 2 == 1) ? v[n / 2] : (v[n / 2 - 1] + v[n / 2]) / 2.0L;
    return {v.front(), med, v.back()};
}

std::string format_scientific(long double value) {
    std::ostringstream out;
    out << std::setprecision(std::numeric_limits<double>::max_digits10) << std::scientific << value;
    return out.str();
}

void print_counter(const char* label, const CounterSummary& s) {
    std::cout << label << ": [" << s.min << ", " << s.median << ", " << s.max << "]\n";
}
void print_value(const char* label, const ValueSummary& s) {
    std::cout << label << ": [" << s.min << ", " << s.median << ", " << s.max << "]\n";
}

// print_collapse_summary, reproducer.cpp:8150-8171
void print_collapse_summary(const std::vector<wr_collapse_state>& cells) {
    const wr_collapse_state& rep = cells.front();
    if (cells.size() == 1) {
        std::cout << "representative cell completed steps: " << rep.completed_steps << "\n";
        std::cout << "representative cell physical time: " << format_scientific(rep.time) << "\n";
        std::cout << "representative cell density driver: " << rep.density_driver << "\n";
        return;
    }
    std::vector<long double> steps, times, drivers;
    for (const auto& c : cells) {
        steps.push_back(static_cast<long double>(c.completed_steps));
        times.push_back(static_cast<long double>(c.time));
        drivers.push_back(static_cast<long double>(c.density_driver));
    }
    print_value("cell completed steps", summarize_value(steps));
    const ValueSummary t = summarize_value(times);
    std::cout << "cell physical time: [" << format_scientific(t.min) << ", " << format_scientific(t.median) << ", "
              << format_scientific(t.max) << "]\n";
    print_value("cell density driver", summarize_value(drivers));
}

// print_stats, reproducer.cpp:8173-8199
void print_stats(const std::vector<wr_collapse_state>& cells) {
    if (cells.size() == 1) {
        const wr_integrator_stats& s = cells.front().stats;
        std::cout << "ROS2S internal steps: " << s.internal_steps << "\n";
        std::cout << "ROS2S rhs calls: " << s.rhs_calls << "\n";
        std::cout << "ROS2S jacobian calls: " << s.jacobian_calls << "\n";
        std::cout << "ROS2S decompositions: " << s.decompositions << "\n";
        std::cout << "ROS2S linear solves: " << s.linear_solves << "\n";
        std::cout << "ROS2S accepted/rejected: " << s.accepted_steps << "/" << s.rejected_steps << "\n\n";
        return;
    }
    auto col = [&](uint64_t wr_integrator_stats::*f) {
        std::vector<uint64_t> v;
        v.reserve(cells.size());
        for (const auto& c : cells) v.push_back(c.stats.*f);
        return summarize_counter(std::move(v));
    };
    print_counter("ROS2S internal steps", col(&wr_integrator_stats::internal_steps));
    print_counter("ROS2S rhs calls", col(&wr_integrator_stats::rhs_calls));
    print_counter("ROS2S jacobian calls", col(&wr_integrator_stats::jacobian_calls));
    print_counter("ROS2S decompositions", col(&wr_integrator_stats::decompositions));
    print_counter("ROS2S linear solves", col(&wr_integrator_stats::linear_solves));
    const CounterSummary a = col(&wr_integrator_stats::accepted_steps);
    const CounterSummary r = col(&wr_integrator_stats::rejected_steps);
    std::cout << "ROS2S accepted/rejected: [" << a.min << "/" << r.min << ", " << a.median << "/" << r.median << ", "
              << a.max << "/" << r.max << "]\n\n";
}

void print_usage(const char* program) {
    std::cerr << "usage: " << program
              << " [--grid N] [--perturb|--no-perturb]"
                 " [--compare-final-state FILE|--no-compare-final-state]"
                 " [--driver-policy gridwide-independent|legacy-local|gridwide-cta32]"
                 " [--write-final-state FILE] [--math portable|cuda]\n";
}

bool parse_positive_int(const char* text, int& value) {  // :8201-8211
    errno = 0;
    char* end = nullptr;
    const long parsed = std::strtol(text, &end, 10);
    if (errno != 0 || end == text || *end != '\0' || parsed <= 0 || parsed > std::numeric_limits<int>::max())
        return false;
    value = static_cast<int>(parsed);
    return true;
}

bool parse_args(int argc, char** argv, Options& o) {  // :8229-8277
    for (int i = 1; i < argc; ++i) {
        const std::string_view arg{argv[i]};
        if (arg == "--help" || arg == "-h") {
            o.show_help = true;
            return true;
        }
        if (arg == "--grid") {
            if (i + 1 >= argc || !parse_positive_int(argv[++i], o.grid_dim)) {
                print_usage(argv[0]);
                return false;
            }
            continue;
        }
        if (arg == "--perturb") {
            o.perturb = true;
            continue;
        }
        if (arg == "--no-perturb") {
            o.perturb = false;
            continue;
        }
        if (arg == "--compare-final-state") {
            if (i + 1 >= argc) {
                print_usage(argv[0]);
                return false;
            }
            o.compare_path = argv[++i];
            continue;
        }
        if (arg == "--no-compare-final-state") {
            o.compare_path.clear();
            continue;
        }
        if (arg == "--math") {
            if (i + 1 >= argc) {
                print_usage(argv[0]);
                return false;
            }
            const std::string_view m{argv[++i]};
            if (m == "portable") {
                o.math = WR_MATH_PORTABLE;
            } else if (m == "cuda") {
                o.math = WR_MATH_CUDA;
            } else {
                print_usage(argv[0]);
                return false;
            }
            continue;
        }
        if (arg == "--driver-policy") {
            if (i + 1 >= argc) {
                print_usage(argv[0]);
                return false;
            }
            const std::string_view p{argv[++i]};
            if (p == "gridwide-independent") {
                o.policy = WR_POLICY_GRIDWIDE_INDEPENDENT;
            } else if (p == "legacy-local") {
                o.policy = WR_POLICY_LEGACY_LOCAL;
            } else if (p == "gridwide-cta32") {
                o.policy = WR_POLICY_GRIDWIDE_CTA32;
            } else {
                print_usage(argv[0]);
                return false;
            }
            continue;
        }
        if (arg == "--write-final-state") {
            if (i + 1 >= argc || argv[i + 1][0] == '\0') {
                print_usage(argv[0]);
                return false;
            }
            o.write_path = argv[++i];
            continue;
        }
        constexpr std::string_view prefix = "--compare-final-state=";
        if (arg.rfind(prefix, 0) == 0) {
            o.compare_path = argv[i] + prefix.size();
            if (o.compare_path.empty()) {
                print_usage(argv[0]);
                return false;
            }
            continue;
        }
        print_usage(argv[0]);
        return false;
    }
    return true;
}

wr_packed_final_state make_packed(const wr_collapse_state& s, int cell, int grid) {  // :8289-8305
    wr_packed_final_state p{};
    p.cell = cell;
    p.i = cell % grid;
    p.j = (cell / grid) % grid;
    p.k = cell / (grid * grid);
    p.completed_steps = s.completed_steps;
    p.time = s.time;
    p.density_driver = s.density_driver;
    p.rho = s.rho;
    p.T = s.T;
    p.e = s.e;
    for (int n = 0; n < WR_NUM_SPECIES; ++n) p.xn[n] = s.xn[n];
    return p;
}

bool rotate_existing_output(const std::string& path) {  // :8314-8355
    namespace fs = std::filesystem;
    std::error_code ec;
    if (!fs::exists(path, ec)) {
        if (ec) {
            std::cerr << "failed to check final-state output file: " << path << " (" << ec.message() << ")\n";
            return false;
        }
        return true;
    }
    std::random_device seed;
    std::mt19937 gen(seed());
    std::uniform_int_distribution<int> dist(0, kBackupLimit - 1);
    for (int attempt = 0; attempt < kBackupAttempts; ++attempt) {
        std::ostringstream b;
        b << path << ".old." << std::setw(kBackupDigits) << std::setfill('0') << dist(gen);
        const std::string backup = b.str();
        if (fs::exists(backup, ec)) {
            if (ec) {
                std::cerr << "failed to check backup final-state file: " << backup << " (" << ec.message() << ")\n";
                return false;
            }
            continue;
        }
        fs::rename(path, backup, ec);
        if (!ec) {
            std::cout << "existing final states moved to: " << backup << "\n";
            return true;
        }
        std::cerr << "failed to move existing final-state output file from " << path << " to " << backup << " ("
                  << ec.message() << ")\n";
        return false;
    }
    std::cerr << "failed to choose a unique backup filename for: " << path << "\n";
    return false;
}

bool write_final_states(const std::vector<wr_collapse_state>& cells, int grid, const std::string& path) {
    if (!rotate_existing_output(path)) return false;
    std::ofstream out(path, std::ios::binary);
    if (!out) {
        std::cerr << "failed to open final-state output file: " << path << "\n";
        return false;
    }
    for (size_t c = 0; c < cells.size(); ++c) {
        const wr_packed_final_state p = make_packed(cells[c], static_cast<int>(c), grid);
        out.write(reinterpret_cast<const char*>(&p), sizeof p);
        if (!out) {
            std::cerr << "failed to write final-state output file: " << path << "\n";
            return false;
        }
    }
    return true;
}

bool read_final_states(const std::string& path, size_t expected, std::vector<wr_packed_final_state>& recs) {
    std::ifstream in(path, std::ios::binary | std::ios::ate);
    if (!in) {
        std::cerr << "failed to open final-state comparison file: " << path << "\n";
        return false;
    }
    const auto size = in.tellg();
    if (size < 0) {
        std::cerr << "failed to determine size of final-state comparison file: " << path << "\n";
        return false;
    }
    const auto bytes = static_cast<uintmax_t>(size);
    const auto want = static_cast<uintmax_t>(expected) * sizeof(wr_packed_final_state);
    if (bytes != want) {
        std::cerr << "final-state comparison file has " << bytes << " bytes, expected " << want << " bytes ("
                  << expected << " packed records of " << sizeof(wr_packed_final_state) << " bytes)\n";
        return false;
    }
    recs.resize(expected);
    in.seekg(0);
    in.read(reinterpret_cast<char*>(recs.data()), static_cast<std::streamsize>(want));
    if (!in && want != 0) {
        std::cerr << "failed to read final-state comparison file: " << path << "\n";
        return false;
    }
    return true;
}

bool nearly_equal(double v, double r, double rtol, double atol) { return std::abs(v - r) <= atol + rtol * std::abs(r); }
long double relative_error(double v, double r, double atol) {
    const double denom = std::max(std::abs(r), atol);
    return static_cast<long double>(std::abs(v - r) / denom);
}
std::string fmt(double v) { return format_scientific(static_cast<long double>(v)); }

std::string csv_escape(const std::string& v) {
    if (v.find_first_of(",\"\n\r") == std::string::npos) return v;
    std::string e = "\"";
    for (char ch : v) {
        if (ch == '"') e.push_back('"');
        e.push_back(ch);
    }
    e.push_back('"');
    return e;
}

struct Failure {
    int32_t cell, i, j, k;
    std::string field, actual, reference, rel, rtol, atol;
};

// compare_final_states + compare_final_states_from_file, reproducer.cpp:8416-8578
bool compare_from_file(const std::vector<wr_collapse_state>& cells, int grid, const std::string& path) {
    std::vector<wr_packed_final_state> ref;
    if (!read_final_states(path, cells.size(), ref)) return false;
    bool pass = true;
    long double max_d = 0, max_nd = 0, max_th = 0, max_rho = 0;
    std::string first;
    std::vector<Failure> fails;
    for (size_t ci = 0; ci < cells.size(); ++ci) {
        const wr_packed_final_state a = make_packed(cells[ci], static_cast<int>(ci), grid);
        const wr_packed_final_state& x = ref[ci];
        const bool meta = a.cell == x.cell && a.i == x.i && a.j == x.j && a.k == x.k && a.completed_steps == x.completed_steps;
        if (!meta && first.empty()) {
            std::ostringstream m;
            m << "metadata mismatch at cell " << ci << " (actual cell/i/j/k/steps " << a.cell << "/" << a.i << "/" << a.j
              << "/" << a.k << "/" << a.completed_steps << ", reference " << x.cell << "/" << x.i << "/" << x.j << "/"
              << x.k << "/" << x.completed_steps << ")";
            first = m.str();
        }
        pass = pass && meta;
        auto meta_fail = [&](const char* f, int32_t av, int32_t rv) {
            fails.push_back({a.cell, a.i, a.j, a.k, f, std::to_string(av), std::to_string(rv), "", "", ""});
        };
        if (a.cell != x.cell) meta_fail("cell", a.cell, x.cell);
        if (a.i != x.i) meta_fail("i", a.i, x.i);
        if (a.j != x.j) meta_fail("j", a.j, x.j);
        if (a.k != x.k) meta_fail("k", a.k, x.k);
        if (a.completed_steps != x.completed_steps) meta_fail("completed_steps", a.completed_steps, x.completed_steps);
        for (int n = 0; n < WR_NUM_SPECIES; ++n) {
            const double v = a.xn[n], r = x.xn[n];
            const long double rel = relative_error(v, r, kAtolSpec);
            long double& mx = is_deuterium_bearing(n) ? max_d : max_nd;
            mx = std::max(mx, rel);
            if (is_deuterium_bearing(n)) continue;
            const bool ok = nearly_equal(v, r, kSpeciesRtol[n], kAtolSpec);
            if (!ok && first.empty()) {
                std::ostringstream m;
                m << "species " << kSpecNames[n] << " mismatch at cell " << ci << " (actual " << format_scientific(v)
                  << ", reference " << format_scientific(r) << ", relative error " << format_scientific(rel)
                  << ", rtol " << kSpeciesRtol[n] << ", atol " << kAtolSpec << ")";
                first = m.str();
            }
            pass = pass && ok;
            if (!ok)
                fails.push_back({a.cell, a.i, a.j, a.k, kSpecNames[n], fmt(v), fmt(r), format_scientific(rel),
                                 fmt(kSpeciesRtol[n]), fmt(kAtolSpec)});
        }
        const long double trel = relative_error(a.T, x.T, kAtolSpec);
        const long double erel = relative_error(a.e, x.e, kAtolEnergy);
        const long double rrel = relative_error(a.rho, x.rho, kAtolSpec);
        max_th = std::max(max_th, std::max(trel, erel));
        max_rho = std::max(max_rho, rrel);
        const bool tok = nearly_equal(a.T, x.T, kThermoRtol, kAtolSpec);
        const bool eok = nearly_equal(a.e, x.e, kThermoRtol, kAtolEnergy);
        const bool rok = nearly_equal(a.rho, x.rho, kRtolSpec, kAtolSpec);
        if ((!tok || !eok || !rok) && first.empty()) {
            std::ostringstream m;
            m << "thermodynamic mismatch at cell " << ci << " (T rel " << format_scientific(trel) << ", e rel "
              << format_scientific(erel) << ", rho rel " << format_scientific(rrel) << ")";
            first = m.str();
        }
        pass = pass && tok && eok && rok;
        if (!tok) fails.push_back({a.cell, a.i, a.j, a.k, "T", fmt(a.T), fmt(x.T), format_scientific(trel), fmt(kThermoRtol), fmt(kAtolSpec)});
        if (!eok) fails.push_back({a.cell, a.i, a.j, a.k, "e", fmt(a.e), fmt(x.e), format_scientific(erel), fmt(kThermoRtol), fmt(kAtolEnergy)});
        if (!rok) fails.push_back({a.cell, a.i, a.j, a.k, "rho", fmt(a.rho), fmt(x.rho), format_scientific(rrel), fmt(kRtolSpec), fmt(kAtolSpec)});
    }
    std::cout << "final-state comparison file: " << path << "\n";
    std::cout << "final-state comparison: " << (pass ? "PASS" : "FAIL") << " (max deuterium-bearing species rel error "
              << format_scientific(max_d) << ", max non-deuterium-bearing species rel error " << format_scientific(max_nd)
              << ", max thermodynamic rel error " << format_scientific(max_th) << ", max rho rel error "
              << format_scientific(max_rho) << ")\n";
    if (!pass && !first.empty()) std::cout << "first comparison failure: " << first << "\n";
    if (!pass && !fails.empty()) {
        std::stable_sort(fails.begin(), fails.end(), [](const Failure& l, const Failure& r) { return l.cell < r.cell; });
        const std::string csv = std::string("final_state_comparison_failures_") + kBackend + ".csv";
        std::ofstream out(csv);
        if (!out) {
            std::cerr << "failed to open comparison-failures CSV file: " << csv << "\n";
            return false;
        }
        out << "cell,i,j,k,field,actual,reference,relative_error,rtol,atol\n";
        for (const auto& f : fails) {
            out << f.cell << ',' << f.i << ',' << f.j << ',' << f.k << ',' << csv_escape(f.field) << ','
                << csv_escape(f.actual) << ',' << csv_escape(f.reference) << ',' << csv_escape(f.rel) << ','
                << csv_escape(f.rtol) << ',' << csv_escape(f.atol) << '\n';
            if (!out) {
                std::cerr << "failed to write comparison-failures CSV file: " << csv << "\n";
                return false;
            }
        }
    }
    return pass;
}

// Manifest sidecar of --write-final-state: what produced the records, so a
// comparison can refuse files from a different program or policy (the Mojo
// reference writes format, cell count, policy and source hashes,
// reproducer.mojo:3283-3308).
const char* policy_name(int policy) {
    return policy == WR_POLICY_LEGACY_LOCAL ? "legacy-local"
           : policy == WR_POLICY_GRIDWIDE_CTA32 ? "gridwide-cta32"
                                                : "gridwide-independent";
}

std::string manifest_contents(int num_cells, const Options& o) {
    std::ostringstream m;
    m << "format=packed-final-state-v1\n"
      << "cell_count=" << num_cells << "\n"
      << "policy=" << policy_name(o.policy) << "-v1\n"
      << "perturbations=" << (o.perturb ? "enabled" : "disabled") << "\n"
      << "math=" << (o.math == WR_MATH_CUDA ? "cuda" : "portable") << "\n"
      << "program=reproducer_gb300\n";
    return m.str();
}

bool write_with_manifest(const std::vector<wr_collapse_state>& cells, int grid, const std::string& path,
                         const Options& o) {
    namespace fs = std::filesystem;
    std::error_code ec;
    const std::string sidecar = path + ".manifest";
    if (fs::exists(path, ec) || fs::exists(sidecar, ec)) {
        std::cerr << "refusing to overwrite final-state output: " << path << "\n";
        return false;
    }
    std::ofstream out(path, std::ios::binary);
    if (!out) {
        std::cerr << "failed to open final-state output file: " << path << "\n";
        return false;
    }
    for (size_t c = 0; c < cells.size(); ++c) {
        const wr_packed_final_state p = make_packed(cells[c], static_cast<int>(c), grid);
        out.write(reinterpret_cast<const char*>(&p), sizeof p);
    }
    out.close();
    std::ofstream man(sidecar);
    man << manifest_contents(static_cast<int>(cells.size()), o);
    if (!out || !man) {
        std::cerr << "failed to write final-state output: " << path << "\n";
        return false;
    }
    return true;
}

void print_state(const wr_collapse_state& s) {  // :8279-8287
    std::cout << "rho: " << s.rho << "\n";
    std::cout << "T: " << s.T << "\n";
    std::cout << "Eint: " << s.e << "\n";
    for (int n = 0; n < WR_NUM_SPECIES; ++n) std::cout << kSpecNames[n] << ": " << s.xn[n] << "\n";
}

}  // namespace

int main(int argc, char** argv) {  // reproducer.cpp:8591-8702
    std::cout << std::setprecision(std::numeric_limits<double>::max_digits10);
    const auto finish = [](bool pass, bool emit) {
        std::cerr.flush();
        if (emit) std::cout << "\n" << (pass ? "PASS" : "FAIL") << "\n";
        return pass ? 0 : 1;
    };
    Options o;
    if (!parse_args(argc, argv, o)) return finish(false, false);
    if (o.show_help) {
        print_usage(argv[0]);
        return finish(true, false);
    }
    const long long cells_ll = static_cast<long long>(o.grid_dim) * o.grid_dim * o.grid_dim;
    if (cells_ll <= 0 || cells_ll > std::numeric_limits<int>::max()) {
        std::cerr << "grid dimension is too large: " << o.grid_dim << "\n";
        return finish(false, false);
    }
    const int num_cells = static_cast<int>(cells_ll);
    std::vector<wr_collapse_state> cells(static_cast<size_t>(num_cells));
    wr_collapse_state init;
    wr_make_collapse_state(&init);
    std::fill(cells.begin(), cells.end(), init);

    int cgs = 0;
    const auto start = std::chrono::steady_clock::now();
    int result = WR_SUCCESS;
    {
        wr_ctx* ctx = nullptr;
        int device = 0;
        result = wr_create(num_cells, device, o.math, &ctx);
        if (result == WR_SUCCESS) result = wr_set_policy(ctx, o.policy);
        if (result == WR_SUCCESS) result = wr_upload(ctx, cells.data());
        if (result == WR_SUCCESS) result = wr_run(ctx, o.perturb ? 1 : 0, &cgs);
        if (ctx) {
            const int rc = wr_download(ctx, cells.data());
            if (rc != WR_SUCCESS && result == WR_SUCCESS) result = rc;
            wr_destroy(ctx);
        }
        if (result != WR_SUCCESS) {
            const char* err = wr_last_error();
            std::cerr << "ROS2S failed on " << kBackend << " with code " << result;
            if (err && *err) std::cerr << " (" << err << ")";
            std::cerr << "\n";
        }
    }
    const auto end = std::chrono::steady_clock::now();
    const double elapsed = std::chrono::duration<double>(end - start).count();
    if (result != WR_SUCCESS) return finish(false, false);

    std::cout << "Primordial chemistry collapse grid with ROS2S\n";
    std::cout << "grid: " << o.grid_dim << "^3 (" << num_cells << " cells)\n";
    std::cout << "perturbations: " << (o.perturb ? "enabled" : "disabled") << "\n";
    // the reference's structured CUDA build prints gridwide-structured-cta32
    // (reproducer.cpp:8666-8667)
    std::cout << "driver policy: "
              << (o.policy == WR_POLICY_GRIDWIDE_CTA32 ? "gridwide-structured-cta32" : policy_name(o.policy)) << "\n";
    std::cout << "completed global collapse steps: " << cgs << "\n";
    print_collapse_summary(cells);
    std::cout << "wall time: " << elapsed << " s\n";
    print_stats(cells);

    bool pass = true, done = false;
    if (!o.compare_path.empty()) {
        done = true;
        pass = compare_from_file(cells, o.grid_dim, o.compare_path);
    }
    if (!o.write_path.empty()) {
        if (!write_with_manifest(cells, o.grid_dim, o.write_path, o)) return finish(false, done);
        std::cout << "final states written: " << o.write_path << " (+ .manifest)\n";
    }
    if (o.grid_dim > 1) {
        std::ostringstream name;
        name << "final_states_grid" << o.grid_dim << "_" << kBackend << ".bin";
        if (!write_final_states(cells, o.grid_dim, name.str())) return finish(false, done);
        std::cout << "final states: " << name.str() << " (" << cells.size() << " packed records, "
                  << sizeof(wr_packed_final_state) << " bytes each)\n";
    } else {
        print_state(cells.front());
    }
    return finish(pass, done);
}
