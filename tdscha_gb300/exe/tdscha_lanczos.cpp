// tdscha-lanczos-gb300: the input-file Lanczos program on the GPU.
//
// Reads the files Lanczos.prepare_input_files writes (<root>.json, .X.dat,
// .Y.dat, .freqs, .rho, .psi, .ndegs, .blockid, .block<i>, .symsb<i>;
// Modules/DynamicalLanczos.py:873-975), runs the bi-Lanczos of the reference's
// MPI program (CModules/Lanczos.cpp:540-820: L q and L^T p each step, plain
// normalisation of the start vector) through libtdscha_gb300, and writes what
// that program writes and load_from_input_files reads back (:978-1057):
// <root>.abc ("a\tb\tc" per step, the last a alone on convergence),
// <root>.qbasis.out / .pbasis.out (one vector per line) and <root>.snorm.out.
// The json keys "restart" / "step_done" continue a run from those files
// (Lanczos.cpp:60-67, :181-226).
//
//   tdscha-lanczos-gb300 <root> [--precision fp64|mixed] [--reorth] [--chunk K]
//
// Host-only C++: every GPU operation goes through the library's C ABI.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "tdscha_gb300.h"

namespace {

// Flat view of a JSON document: every scalar under its dotted key path.
class FlatJson {
  public:
    explicit FlatJson(const std::string &text) : s_(text), i_(0) {
        skip();
        value("");
    }
    bool has(const std::string &k) const { return v_.count(k) != 0; }
    const std::string &raw(const std::string &k) const {
        auto it = v_.find(k);
        if (it == v_.end()) throw std::runtime_error("json: missing key " + k);
        return it->second;
    }
    double num(const std::string &k) const { return std::stod(raw(k)); }
    bool flag(const std::string &k) const {
        const std::string &r = raw(k);
        if (r == "true") return true;
        if (r == "false") return false;
        return std::stod(r) != 0;
    }

  private:
    void skip() { while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) ++i_; }
    void expect(char c) {
        skip();
        if (i_ >= s_.size() || s_[i_] != c) throw std::runtime_error(std::string("json: expected ") + c);
        ++i_;
    }
    std::string str() {
        expect('"');
        std::string out;
        while (i_ < s_.size() && s_[i_] != '"') {
            if (s_[i_] == '\\' && i_ + 1 < s_.size()) ++i_;
            out += s_[i_++];
        }
        expect('"');
        return out;
    }
    void value(const std::string &path) {
        skip();
        if (i_ >= s_.size()) throw std::runtime_error("json: truncated");
        char c = s_[i_];
        if (c == '{') {
            ++i_;
            skip();
            if (s_[i_] == '}') { ++i_; return; }
            while (true) {
                std::string k = str();
                expect(':');
                value(path.empty() ? k : path + "." + k);
                skip();
                if (s_[i_] == ',') { ++i_; continue; }
                expect('}');
                return;
            }
        } else if (c == '[') {      // arrays are not used by the input format: skip
            int depth = 0;
            do {
                if (s_[i_] == '[') ++depth;
                if (s_[i_] == ']') --depth;
                ++i_;
            } while (depth > 0 && i_ < s_.size());
        } else if (c == '"') {
            v_[path] = str();
        } else {
            size_t j = i_;
            while (j < s_.size() && s_[j] != ',' && s_[j] != '}' && s_[j] != ']' &&
                   !std::isspace((unsigned char)s_[j]))
                ++j;
            v_[path] = s_.substr(i_, j - i_);
            i_ = j;
        }
    }
    std::string s_;
    size_t i_;
    std::map<std::string, std::string> v_;
};

std::string slurp(const std::string &f) {
    std::ifstream in(f);
    if (!in) throw std::runtime_error("cannot open " + f);
    std::stringstream ss;
    ss << in.rdbuf();
    return ss.str();
}

template <class T>
std::vector<T> read_values(const std::string &f, size_t n) {
    std::ifstream in(f);
    if (!in) throw std::runtime_error("cannot open " + f);
    std::vector<T> v(n);
    for (size_t k = 0; k < n; ++k)
        if (!(in >> v[k])) throw std::runtime_error("not enough values in " + f);
    return v;
}

void check(int rc, const char *what) {
    if (rc != TDSCHA_OK)
        throw std::runtime_error(std::string(what) + ": " + tdscha_last_error());
}

void usage() {
    std::cout << "LANCZOS CALCULATOR PROGRAM (GB300)\n"
                 "Usage: tdscha-lanczos-gb300 <rootname> [--precision fp64|mixed] [--reorth] "
                 "[--chunk K]\n"
                 "<rootname> is the name given to Lanczos.prepare_input_files.\n";
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 2) {
        usage();
        return EXIT_FAILURE;
    }
    std::string root = argv[1];
    int precision = TDSCHA_PREC_FP64, reorth = 0, chunk = 16;
    for (int a = 2; a < argc; ++a) {
        std::string o = argv[a];
        if (o == "--precision" && a + 1 < argc) {
            std::string p = argv[++a];
            if (p == "mixed") precision = TDSCHA_PREC_MIXED;
            else if (p != "fp64") { usage(); return EXIT_FAILURE; }
        } else if (o == "--reorth") {
            reorth = 1;
        } else if (o == "--chunk" && a + 1 < argc) {
            chunk = std::max(1, std::atoi(argv[++a]));
        } else {
            usage();
            return EXIT_FAILURE;
        }
    }
    tdscha_ctx *ctx = nullptr;
    try {
        FlatJson js(slurp(root + ".json"));
        const double T = js.num("T");
        const int n_steps = (int)js.num("n_steps");
        const bool ignore_v2 = js.flag("ignore_v2"), ignore_v3 = js.flag("ignore_v3"),
                   ignore_v4 = js.flag("ignore_v4");
        int step_done = 0;
        bool restart = false;
        if (js.has("restart")) {
            restart = js.flag("restart");
            step_done = restart ? (int)js.num("step_done") : 0;
        }
        if (step_done >= n_steps) throw std::invalid_argument("n_steps must be greater than step_done");
        const int N = (int)js.num("data.n_configs"), M = (int)js.num("data.n_modes");
        const int n_syms = (int)js.num("data.n_syms"), n_blocks = (int)js.num("data.n_blocks");
        const bool reverse = js.flag("data.reverse");
        const double shift = js.num("data.shift");
        const long P = (long)M + (long)M * (M + 1);

        auto n_deg = read_values<int>(root + ".ndegs", n_blocks);
        auto w = read_values<double>(root + ".freqs", M);
        auto rho = read_values<double>(root + ".rho", N);
        auto psi = read_values<double>(root + ".psi", P);
        auto X = read_values<double>(root + ".X.dat", (size_t)N * M);
        auto Y = read_values<double>(root + ".Y.dat", (size_t)N * M);
        auto bid = read_values<int>(root + ".blockid", M);
        std::vector<int> deg;
        std::vector<double> sym;
        for (int b = 0; b < n_blocks; ++b) {
            auto d = read_values<int>(root + ".block" + std::to_string(b), n_deg[b]);
            deg.insert(deg.end(), d.begin(), d.end());
            auto s = read_values<double>(root + ".symsb" + std::to_string(b),
                                         (size_t)n_syms * n_deg[b] * n_deg[b]);
            sym.insert(sym.end(), s.begin(), s.end());
        }

        const int cap = n_steps + 1;
        std::vector<double> Q((size_t)cap * P), Pb((size_t)cap * P), hist(4 * (size_t)cap + 4, 0.0);
        if (restart) {
            auto abc = read_values<double>(root + ".abc", 3 * (size_t)step_done);
            auto q = read_values<double>(root + ".qbasis.out", (size_t)P * (step_done + 1));
            auto p = read_values<double>(root + ".pbasis.out", (size_t)P * (step_done + 1));
            auto sn = read_values<double>(root + ".snorm.out", step_done + 1);
            std::copy(q.begin(), q.end(), Q.begin());
            std::copy(p.begin(), p.end(), Pb.begin());
            for (int k = 0; k < step_done; ++k) {
                hist[4 * k] = abc[3 * k];
                hist[4 * k + 1] = abc[3 * k + 1];
                hist[4 * k + 2] = abc[3 * k + 2];
            }
            for (int k = 0; k <= step_done; ++k) hist[4 * k + 3] = sn[k];
        } else {
            double nrm = 0;
            for (long j = 0; j < P; ++j) nrm += psi[j] * psi[j];
            nrm = std::sqrt(nrm);
            for (long j = 0; j < P; ++j) Q[j] = Pb[j] = psi[j] / nrm;
            hist[3] = 1;
        }

        check(tdscha_ctx_create(&ctx, M, N, X.data(), Y.data(), w.data(), rho.data(), T, n_syms,
                                n_blocks, n_deg.data(), deg.data(), sym.data(), bid.data(),
                                precision == TDSCHA_PREC_MIXED),
              "tdscha_ctx_create");
        // the MPI program runs the non-Wigner representation
        check(tdscha_ctx_set_options(ctx, 0, ignore_v2, ignore_v3, ignore_v4, reverse, shift),
              "tdscha_ctx_set_options");

        std::ios::openmode mode = std::ios::out | (restart ? std::ios::app : std::ios::trunc);
        std::ofstream fabc(root + ".abc", mode), fq(root + ".qbasis.out", mode),
            fp(root + ".pbasis.out", mode), fs(root + ".snorm.out", mode);
        for (auto *f : {&fabc, &fq, &fp, &fs}) *f << std::scientific << std::setprecision(16);
        auto write_row = [&](std::ofstream &f, const std::vector<double> &B, int k) {
            for (long j = 0; j < P; ++j) f << B[(size_t)k * P + j] << " ";
            f << "\n";
        };
        if (!restart) {
            write_row(fq, Q, 0);
            write_row(fp, Pb, 0);
            fs << hist[3] << "\n";
        }
        int step = step_done;
        bool converged = false;
        while (step < n_steps && !converged) {
            int todo = std::min(chunk, n_steps - step);
            int done = 0, conv = 0;
            check(tdscha_lanczos_run_hostbuf(ctx, Q.data(), Pb.data(), cap, step, todo, 0, precision,
                                             reorth, hist.data(), &done, &conv),
                  "tdscha_lanczos_run");
            for (int k = step; k < step + done; ++k) {
                if (conv && k == step + done - 1) {
                    fabc << hist[4 * k] << "\n";
                    std::cout << "  Converged.\n The last a coefficient is " << std::scientific
                              << std::setprecision(16) << hist[4 * k] << "\n";
                    break;
                }
                fabc << hist[4 * k] << "\t" << hist[4 * k + 1] << "\t" << hist[4 * k + 2] << "\n";
                fs << hist[4 * (k + 1) + 3] << "\n";
                write_row(fq, Q, k + 1);
                write_row(fp, Pb, k + 1);
                std::cout << "a_" << k << " = " << std::scientific << std::setprecision(16)
                          << hist[4 * k] << "\nb_" << k << " = " << hist[4 * k + 1] << "\nc_" << k
                          << " = " << hist[4 * k + 2] << "\n";
            }
            for (auto *f : {&fabc, &fq, &fp, &fs}) f->flush();
            converged = conv != 0;
            step += done;
            if (done < todo && !converged) break;
        }
        std::cout << "I'm done with the calculation!" << std::endl;
        tdscha_ctx_destroy(ctx);
    } catch (const std::exception &e) {
        std::cerr << "tdscha-lanczos-gb300: " << e.what() << std::endl;
        if (ctx) tdscha_ctx_destroy(ctx);
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
