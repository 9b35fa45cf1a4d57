// Host model of a reaction network and its packed device descriptor.
//
// A reaction is a rate constant, a multiply sequence of (species, order)
// factors and the non-zero entries of its species-difference vector.  The
// multiply sequence reproduces Rate::rate of rebop's run-time API
// (src/gillespie.rs:71-90): for Rate::lma the non-zero exponents in species
// order, for Rate::lma_sparse the pairs in the order the caller gave them.
// Networks lowered from define_system! text keep the macro's arithmetic
// instead (src/gillespie_macro.rs:106, :133-171), flagged by macro_mode.
#pragma once

#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

namespace rbg {

struct Factor {
    int32_t species;
    int32_t order;
};

struct JumpEntry {
    int32_t species;
    int64_t delta;
};

// Tiny expression tree for define_system! rate expressions (`@ k`, `@ 0.1`,
// `@ k1 / k2`): evaluated on the host whenever a parameter changes.
struct RateExpr {
    enum Op : int32_t { Const, Param, Neg, Add, Sub, Mul, Div };
    Op op = Const;
    double value = 0.0;
    int32_t param = -1;
    std::shared_ptr<RateExpr> a, b;
    double eval(const std::vector<double> &params) const;
};

// Rate::Expr of the run-time API (src/expr.rs:8-39) as a postfix program:
// each word is op | argument << 8, the argument a constant index (ExConst) or
// a species index (ExSpecies).
enum ExOp : int32_t { ExConst = 0, ExSpecies, ExNeg, ExAdd, ExSub, ExMul, ExDiv, ExPow, ExMax, ExMin, ExExp };
constexpr int kExMaxDepth = 16;  // evaluation stack of the device interpreter (kExprMaxDepth)

struct Reaction {
    double rate = 0.0;
    std::shared_ptr<RateExpr> rate_expr;  // DSL networks only
    std::vector<int32_t> ex_code;         // Rate::Expr: the propensity is this program's value
    std::vector<double> ex_const;
    std::vector<Factor> factors;          // propensity multiply sequence
    std::vector<JumpEntry> jump;          // non-zero differences, ascending species
    std::string name;
};

// Flat arrays the kernels read (row-major, padded to P factors and Q jump
// entries per reaction; padding factors have order 0, padding jumps delta 0).
struct Packed {
    int32_t S = 0, R = 0, P = 1, Q = 1;
    int32_t macro_mode = 0;
    int32_t max_order = 0;
    std::vector<double> rate;       // [R]
    std::vector<int32_t> fac_sp;    // [R*P]
    std::vector<int32_t> fac_ord;   // [R*P]
    std::vector<int32_t> jmp_sp;    // [R*Q]
    std::vector<int64_t> jmp_d;     // [R*Q]
    // Rate::Expr programs: reaction r's words are ex_code[ex_off[r] .. ex_off[r+1])
    // (empty for mass action), constant arguments index ex_const.
    int32_t has_expr = 0;
    std::vector<int32_t> ex_off;    // [R+1]
    std::vector<int32_t> ex_code;
    std::vector<double> ex_const;
};

struct DeviceNet;  // engine.cpp

struct Network {
    int32_t n_species = 0;
    std::vector<Reaction> reactions;
    bool macro_mode = false;
    std::string name;
    std::vector<std::string> species_names;
    std::vector<std::string> param_names;
    std::vector<double> param_values;
    uint64_t version = 1;  // bumped on every change; device copies compare it

    mutable std::mutex mu;
    mutable std::unique_ptr<DeviceNet> dev;  // lazily uploaded descriptor + buffers

    Network();
    ~Network();

    // Rate::lma / Rate::lma_sparse + differences -> Reaction; returns an
    // error message ("" on success) mirroring add_reaction's asserts.
    std::string add_lma(double rate, const uint32_t *exps, int32_t n_exps, const int64_t *diffs,
                        int32_t n_diffs);
    std::string add_lma_sparse(double rate, const uint32_t *species, const uint32_t *exps,
                               int32_t n_pairs, const int64_t *diffs, int32_t n_diffs);
    // Rate::expr(program) + differences (gillespie.rs:33-35, :88)
    std::string add_expr(const int32_t *code, int32_t n_code, const double *consts, int32_t n_consts,
                         const int64_t *diffs, int32_t n_diffs);
    std::string set_param(const std::string &pname, double value);
    void refresh_rates();
    Packed pack() const;
};

// define_system! body -> Network (macro_mode = true); "" on success.
std::string parse_dsl(const std::string &text, Network &net);

}  // namespace rbg
