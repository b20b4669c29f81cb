// See cmdline.h. Own implementation of the reference's option grammar.
#include "cmdline.h"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <filesystem>
#include <functional>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>

namespace nqes_cli {

namespace {

std::string lower(std::string s) {
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return char(std::tolower(c)); });
    return s;
}

template <class T> std::string to_str(const T &v) {
    std::ostringstream ss;
    ss << std::boolalpha << v;
    return ss.str();
}

struct Opt {
    std::vector<std::string> keys;
    std::string help;
    bool flag = false;
    bool required = false;
    std::string default_str;   // shown in the help text
    std::string allowed;       // enum values, for the help text
    std::function<void(const std::string &)> convert;  // throws invalid_argument / runtime_error
    bool set = false;
    std::string error;

    std::string keys_str() const {
        std::string s;
        for (size_t t = 0; t < keys.size(); t++) s += (t ? "," : "") + std::string(keys[t].size() > 1 ? "--" : "-") + keys[t];
        return s;
    }
    void apply(const std::string &v) {
        set = true;
        try {
            convert(v);
        } catch (const std::invalid_argument &) {
            error = "Invalid argument, could not convert \"" + v + "\" for " + keys_str() + " (" + help + ")";
        } catch (const std::out_of_range &) {
            error = "Invalid argument, could not convert \"" + v + "\" for " + keys_str() + " (" + help + ")";
        } catch (const std::runtime_error &e) {
            error = "Invalid argument \"" + v + "\" for " + keys_str() + " (" + help + "). Error: " + e.what();
        }
    }
    std::string info() const {
        std::string s = " [";
        if (!allowed.empty()) s += "allowed: <" + allowed + ">, ";
        if (flag) s += "implicit: \"true\", ";
        s += required ? "required" : "default: " + default_str;
        return s + "]";
    }
};

const char *kModelNames[] = {"ising", "periodicising", "hs", "xxz", "longrange", "trappedion"};

}  // namespace

CmdArgs parse_args(int argc, char **argv, const std::string &welcome, bool with_dump_options) {
    CmdArgs a;
    std::vector<std::shared_ptr<Opt>> opts;
    std::map<std::string, std::shared_ptr<Opt>> by_key;
    auto add = [&](const std::string &keys, const std::string &help, bool required, const std::string &dflt,
                   std::function<void(const std::string &)> conv, bool flag = false) {
        auto o = std::make_shared<Opt>();
        std::stringstream ks(keys);
        std::string k;
        while (std::getline(ks, k, ',')) o->keys.push_back(k);
        o->help = help;
        o->required = required;
        o->default_str = dflt;
        o->convert = std::move(conv);
        o->flag = flag;
        opts.push_back(o);
        for (auto &kk : o->keys) by_key[kk] = o;
        return o;
    };
    auto dbl = [](double &dst) { return [&dst](const std::string &v) { dst = std::stod(v); }; };
    auto integer = [](int &dst) { return [&dst](const std::string &v) { dst = std::stoi(v); }; };
    auto str = [](std::string &dst) { return [&dst](const std::string &v) { dst = v; }; };
    auto boolean = [](bool &dst) {
        return [&dst](const std::string &v) { dst = lower(v) == "true" || v == "1"; };
    };

    auto model = add("model", "Model to simulate", true, "", [&a](const std::string &v) {
        const std::string lv = lower(v);
        for (int t = 0; t < 6; t++)
            if (lv == kModelNames[t]) {
                a.model = Model(t);
                return;
            }
        std::string e = "enum is only accepting [";
        for (int t = 0; t < 6; t++) e += (t ? ", " : "") + std::string(kModelNames[t]);
        throw std::runtime_error(e + "]");
    });
    model->allowed = "ising, periodicising, hs, xxz, longrange, trappedion";
    add("h", "Specify the external field h.", true, "", dbl(a.h));
    add("n,niters", "Specify the number of iterations to perform.", true, "", integer(a.niters));
    add("m,mc-steps-percpu", "Specify the number of Monte Carlo samples per CPU core.", true, "",
        integer(a.mc_steps_percpu));
    add("c,ncpus", "Specify the number of CPU cores to use.", true, "", integer(a.ncpus));
    add("burn-in-steps", "Specify the number of burn-in steps.", false, "64", integer(a.burn_in_steps));
    add("tol", "Specify the stopping tolerance for the per-partile energy.", false, to_str(1e-6), dbl(a.tol));
    add("lrate-init", "Specify the initial learning rate. Learning rate decreases as training goes on.", false,
        to_str(0.1), dbl(a.lrate0));
    add("lrate-decay", "Specify the decay factor of the learning rate, ie. lrate(t) = lrate(0) * f^t.", false,
        to_str(0.99), dbl(a.lratef));
    add("lrate-cutoff", "Specify the minimal value of the learning rate.", false, to_str(0.01), dbl(a.lrate_cutoff));
    add("reglam-init", "Specify the initial value for the lambda used in regulating S_kk.", false, to_str(0.01),
        dbl(a.reglam0));
    add("reglam-decay", "Specify the decay factor for the lambda used in regulating S_kk.", false, to_str(0.9),
        dbl(a.reglam_decay));
    add("reglam-cutoff", "Specify the minimal value for the lambda used in regulating S_kk.", false, to_str(0.001),
        dbl(a.reglam_cutoff));
    add("minres-rtol", "Specify the tolerance of the MINRES-QLP algorithm.", false, to_str(1e-10), dbl(a.minres_rtol));
    add("minres-maxit", "Specify the max number of iterations for the MINRES-QLP algorithm.", false,
        to_str(~0ULL), [&a](const std::string &v) { a.minres_maxit = std::stoul(v); });
    add("seed", "Specify the seed of the RNG.", false, "none", [&a](const std::string &v) { a.seed = std::stoul(v); });
    add("load-rbm", "If specified, the initial RBM weights will be loaded from the given .mat file.", false, "",
        str(a.load_rbm));
    add("load-single-rbm",
        "If specified, the initial weights will be loaded from the given single RBM with spins flipped except for "
        "the first RBM.",
        false, "", str(a.load_single_rbm));
    add("dump-rbm", "If specified, will dump the weights of the RBMs to the file with the given prefix.", false, "",
        str(a.dump_rbm));
    add("throw-fperror", "Throw an exception when a floating point error has occurred.", false, "false",
        boolean(a.throw_fperror), true);
    add("apply-gauge",
        "When dumping the RBM weights, apply the local gauge transformation a_i -> a_i - I PI / 2 for odd i", false,
        "false", boolean(a.apply_gauge), true);
    add("inverse-gauge",
        "When loading RBM weights, apply the inverse gauge transformation a_i -> a_i + I PI / 2 for odd i", false,
        "false", boolean(a.inverse_gauge), true);
    add("correlation-data", "Specify the file name to save the correlation function data.", true, "",
        str(a.correlation_data));
    if (with_dump_options) {
        add("dump-states", "If specified, will dump the states of the RBMs to the file with the given prefix.", false,
            "", str(a.dump_states));
        add("dump-ham", "If specified, will dump the Hamiltonian for each spin config to the file with the given "
                        "prefix.", false, "", str(a.dump_ham));
        add("dump-deriv", "If specified, will dump the derivatives for each spin config to the file with the given "
                          "prefix.", false, "", str(a.dump_deriv));
    }
    add("jmat",
        "Trapped-ion couplings: a MAT file holding the N x N matrix J, or 'synthetic' for the chain "
        "J_ij = |i-j|^-1.2 (default: the compiled-in Jmat/Ising2d_N{N}_alpha1.0.mat).",
        false, "", str(a.jmat));
    add("dump-jmat", "If specified, write the coupling matrix J this run would use to the given .mat file "
                     "(variable J) and exit.", false, "", str(a.dump_jmat));
    add("device", "CUDA device to run on.", false, "0", integer(a.device));
    bool help = false;
    add("?,help", "print help", false, "false", boolean(help), true);

    const std::string program = std::filesystem::path(argv[0]).stem().string();
    std::vector<std::string> params(argv + 1, argv + argc);
    auto is_value = [&](size_t i) {
        return i < params.size() &&
               (params[i].empty() || params[i][0] != '-' || (params[i].size() > 1 && std::isdigit(params[i][1])));
    };
    auto parse_param = [&](size_t &i, const std::string &key, bool is_short, const std::optional<std::string> &eq) {
        auto it = by_key.find(key);
        if (it == by_key.end()) {
            std::cerr << "unrecognised commandline argument: " << key << std::endl;
            return;
        }
        Opt &o = *it->second;
        if (eq) {
            o.apply(*eq);
        } else if (o.flag) {
            o.apply("true");
        } else if (!is_short) {
            if (is_value(i + 1)) {
                o.apply(params[++i]);
            } else {
                o.error = "No value provided for: " + key;
            }
        } else {
            o.error = "No value provided for: " + key;
        }
    };
    auto add_param = [&](size_t &i, size_t start) {
        const size_t eq = params[i].find('=');
        if (eq != std::string::npos)
            parse_param(i, params[i].substr(start, eq - start), false, params[i].substr(eq + 1));
        else
            parse_param(i, params[i].substr(start), false, std::nullopt);
    };
    for (size_t i = 0; i < params.size(); i++) {
        if (is_value(i)) continue;  // this build has no positional arguments
        if (params[i].size() > 1 && params[i][1] == '-') {
            add_param(i, 2);
        } else {
            const size_t j_end = std::min(params[i].size(), params[i].find('=')) - 1;
            for (size_t j = 1; j < j_end; j++) parse_param(i, std::string(1, params[i][j]), true, std::nullopt);
            add_param(i, j_end);
        }
    }
    for (auto &o : opts)
        if (!o->set && o->required && o->error.empty())
            o->error = "Argument missing: " + o->keys_str() + " (" + o->help + ")";
    if (help) {
        std::cout << welcome;
        std::cout << "Usage: " << program << " " << " [options...]" << std::endl;
        std::cout << std::endl << "Options:" << std::endl;
        for (auto &o : opts) std::cout << std::setw(17) << o->keys_str() << " : " << o->help << o->info() << std::endl;
        std::exit(0);
    }
    for (auto &o : opts)
        if (!o->error.empty()) {
            std::cerr << o->error << std::endl;
            std::exit(-1);
        }
    return a;
}

}  // namespace nqes_cli
