// Command-line surface of the drop-in executable.
//
// Reproduces the behaviour of the reference's CmdArgs (code/rbm.cc:900-961)
// as parsed by its argparse header (code/argparse.h:435-551): keyword options
// `--key value`, `--key=value`, `-k value`; a value may look like a negative
// number; flags take no value; case-insensitive enum for --model; defaults;
// missing required options print "Argument missing: <keys> (<help>)" and exit
// with status 255; conversion failures print "Invalid argument ..." and exit
// 255; unknown options print "unrecognised commandline argument: <key>" and
// are ignored; -?/--help prints the usage (after the welcome line) and exits 0.
#pragma once
#include <cstdint>
#include <optional>
#include <string>
#include <vector>

namespace nqes_cli {

enum class Model { Ising, PeriodicIsing, HS, XXZ, LongRange, TrappedIon };

struct CmdArgs {
    Model model = Model::TrappedIon;
    double h = 0;
    int niters = 0, mc_steps_percpu = 0, ncpus = 0;
    int burn_in_steps = 64;
    double tol = 1e-6, lrate0 = 0.1, lratef = 0.99, lrate_cutoff = 0.01;
    double reglam0 = 0.01, reglam_decay = 0.9, reglam_cutoff = 0.001, minres_rtol = 1e-10;
    uint64_t minres_maxit = ~0ULL;
    std::optional<uint64_t> seed;
    std::string load_rbm, load_single_rbm, dump_rbm, correlation_data;
    bool throw_fperror = false, apply_gauge = false, inverse_gauge = false;
    std::string dump_states, dump_ham, dump_deriv;
    // options of this build that the reference does not have
    std::string jmat;  // MAT file with an N×N variable "J", or "synthetic" (replaces the compiled-in Jmat)
    std::string dump_jmat;  // write the J of this run to a MAT file and exit (no device needed)
    int device = 0;
};

// Parses argv; prints and exits on help or errors exactly like the reference.
// `welcome` is printed before the usage text.
CmdArgs parse_args(int argc, char **argv, const std::string &welcome, bool with_dump_options);

}  // namespace nqes_cli
