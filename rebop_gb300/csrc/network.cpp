// Network construction, validation, packing and define_system! lowering.
#include "network.hpp"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>

#include "engine.hpp"
#include "ssa_args.hpp"

namespace rbg {

static_assert(kExMaxDepth == kExprMaxDepth, "expression stack depth");

Network::Network() = default;
Network::~Network() = default;

double RateExpr::eval(const std::vector<double> &params) const {
    switch (op) {
        case Const: return value;
        case Param: return params[param];
        case Neg: return -a->eval(params);
        case Add: return a->eval(params) + b->eval(params);
        case Sub: return a->eval(params) - b->eval(params);
        case Mul: return a->eval(params) * b->eval(params);
        case Div: return a->eval(params) / b->eval(params);
    }
    return std::numeric_limits<double>::quiet_NaN();
}

static std::vector<JumpEntry> jump_from_dense(const int64_t *diffs, int32_t n) {
    std::vector<JumpEntry> j;
    for (int32_t s = 0; s < n; s++)
        if (diffs[s] != 0) j.push_back({s, diffs[s]});
    return j;
}

// add_reaction with Rate::lma: gillespie.rs:225-244 asserts that the exponent
// vector and the difference vector both have one entry per species.
std::string Network::add_lma(double rate, const uint32_t *exps, int32_t n_exps, const int64_t *diffs,
                             int32_t n_diffs) {
    if (n_exps != n_species)
        return "assertion failed: rate exponents length " + std::to_string(n_exps) +
               " != number of species " + std::to_string(n_species);
    if (n_diffs != n_species)
        return "assertion failed: differences length " + std::to_string(n_diffs) +
               " != number of species " + std::to_string(n_species);
    if (n_species > 0 && (!exps || !diffs)) return "null exponent or difference pointer";
    Reaction r;
    r.rate = rate;
    // The dense fold visits species in index order and multiplies nothing
    // for a zero exponent (gillespie.rs:73-78).
    for (int32_t s = 0; s < n_species; s++)
        if (exps[s] > 0) r.factors.push_back({s, (int32_t)exps[s]});
    for (const Factor &f : r.factors)
        if (f.order > (1 << 20)) return "rate exponent too large";
    r.jump = jump_from_dense(diffs, n_diffs);
    reactions.push_back(std::move(r));
    version++;
    return "";
}

// add_reaction with Rate::lma_sparse: every index must name a species
// (gillespie.rs:229-233, the issue-85 assert); pairs keep the caller's order,
// as the sparse arm of Rate::rate multiplies them (gillespie.rs:79-86).
std::string Network::add_lma_sparse(double rate, const uint32_t *species, const uint32_t *exps,
                                    int32_t n_pairs, const int64_t *diffs, int32_t n_diffs) {
    if (n_pairs < 0) return "negative number of rate pairs";
    if (n_pairs > 0 && (!species || !exps)) return "null rate pair pointer";
    for (int32_t p = 0; p < n_pairs; p++)
        if ((int64_t)species[p] >= n_species)
            return "assertion failed: rate species index " + std::to_string(species[p]) +
                   " out of range for " + std::to_string(n_species) + " species";
    if (n_diffs != n_species)
        return "assertion failed: differences length " + std::to_string(n_diffs) +
               " != number of species " + std::to_string(n_species);
    if (n_species > 0 && !diffs) return "null difference pointer";
    Reaction r;
    r.rate = rate;
    for (int32_t p = 0; p < n_pairs; p++) {
        if (exps[p] > (1u << 20)) return "rate exponent too large";
        if (exps[p] > 0) r.factors.push_back({(int32_t)species[p], (int32_t)exps[p]});
    }
    r.jump = jump_from_dense(diffs, n_diffs);
    reactions.push_back(std::move(r));
    version++;
    return "";
}

// add_reaction with Rate::expr: the difference vector has one entry per
// species (gillespie.rs:225-244); the program must be a well-formed postfix
// form of an Expr tree over this network's species.
std::string Network::add_expr(const int32_t *code, int32_t n_code, const double *consts, int32_t n_consts,
                              const int64_t *diffs, int32_t n_diffs) {
    if (n_code < 1 || !code) return "empty rate expression";
    if (n_consts < 0 || (n_consts > 0 && !consts)) return "null expression constants";
    if (n_diffs != n_species)
        return "assertion failed: differences length " + std::to_string(n_diffs) +
               " != number of species " + std::to_string(n_species);
    if (n_species > 0 && !diffs) return "null difference pointer";
    int depth = 0;
    for (int32_t k = 0; k < n_code; k++) {
        const int32_t op = code[k] & 0xff, arg = code[k] >> 8;
        if (op > ExExp) return "unknown expression operation " + std::to_string(op);
        if (op == ExConst && (arg < 0 || arg >= n_consts)) return "expression constant index out of range";
        if (op == ExSpecies && (arg < 0 || arg >= n_species))
            return "expression species index " + std::to_string(arg) + " out of range";
        depth += (op <= ExSpecies) ? 1 : (op == ExNeg || op == ExExp) ? 0 : -1;
        if (depth < 1) return "malformed rate expression";
        if (depth > kExMaxDepth) return "rate expression nests too deeply";
    }
    if (depth != 1) return "malformed rate expression";
    Reaction r;
    r.ex_code.assign(code, code + n_code);
    r.ex_const.assign(consts, consts + n_consts);
    r.jump = jump_from_dense(diffs, n_diffs);
    reactions.push_back(std::move(r));
    version++;
    return "";
}

std::string Network::set_param(const std::string &pname, double value) {
    for (size_t i = 0; i < param_names.size(); i++) {
        if (param_names[i] == pname) {
            param_values[i] = value;
            refresh_rates();
            return "";
        }
    }
    return "unknown parameter '" + pname + "'";
}

void Network::refresh_rates() {
    for (Reaction &r : reactions)
        if (r.rate_expr) r.rate = r.rate_expr->eval(param_values);
    version++;
}

Packed Network::pack() const {
    Packed p;
    p.S = n_species;
    p.R = (int32_t)reactions.size();
    p.macro_mode = macro_mode ? 1 : 0;
    int32_t P = 1, Q = 1;
    for (const Reaction &r : reactions) {
        P = std::max<int32_t>(P, (int32_t)r.factors.size());
        Q = std::max<int32_t>(Q, (int32_t)r.jump.size());
    }
    p.P = P;
    p.Q = Q;
    p.rate.resize(p.R);
    p.fac_sp.assign((size_t)p.R * P, 0);
    p.fac_ord.assign((size_t)p.R * P, 0);
    p.jmp_sp.assign((size_t)p.R * Q, 0);
    p.jmp_d.assign((size_t)p.R * Q, 0);
    p.ex_off.assign((size_t)p.R + 1, 0);
    for (int32_t i = 0; i < p.R; i++) {
        const Reaction &r = reactions[i];
        const int32_t base = (int32_t)p.ex_const.size();
        for (int32_t w : r.ex_code)
            p.ex_code.push_back((w & 0xff) == ExConst ? (ExConst | (((w >> 8) + base) << 8)) : w);
        p.ex_const.insert(p.ex_const.end(), r.ex_const.begin(), r.ex_const.end());
        p.ex_off[(size_t)i + 1] = (int32_t)p.ex_code.size();
        if (!r.ex_code.empty()) p.has_expr = 1;
        p.rate[i] = r.rate;
        for (size_t k = 0; k < r.factors.size(); k++) {
            p.fac_sp[(size_t)i * P + k] = r.factors[k].species;
            p.fac_ord[(size_t)i * P + k] = r.factors[k].order;
            p.max_order = std::max(p.max_order, r.factors[k].order);
        }
        for (size_t k = 0; k < r.jump.size(); k++) {
            p.jmp_sp[(size_t)i * Q + k] = r.jump[k].species;
            p.jmp_d[(size_t)i * Q + k] = r.jump[k].delta;
        }
    }
    return p;
}

// ---------------------------------------------------------------- DSL ----
// Grammar of define_system! (src/gillespie_macro.rs:50-58):
//   params*  ';'  Name '{' species (',' species)* '}'
//   ( rname ':' side '=>' side '@' rate )*
//   side := [ [int] ident ( '+' [int] ident )* ]
// Identifiers may hold any non-ASCII UTF-8 bytes (the Vilar model names its
// parameters with Greek letters).

namespace {

struct Tok {
    enum Kind { Ident, Number, Punct, End } kind;
    std::string text;
    size_t pos;
};

bool ident_start(unsigned char c) { return std::isalpha(c) || c == '_' || c >= 0x80; }
bool ident_char(unsigned char c) { return std::isalnum(c) || c == '_' || c >= 0x80; }

std::string tokenize(const std::string &s, std::vector<Tok> &out) {
    size_t i = 0, n = s.size();
    while (i < n) {
        unsigned char c = s[i];
        if (std::isspace(c)) { i++; continue; }
        if (c == '/' && i + 1 < n && s[i + 1] == '/') {  // line comment
            while (i < n && s[i] != '\n') i++;
            continue;
        }
        size_t st = i;
        if (ident_start(c)) {
            while (i < n && ident_char((unsigned char)s[i])) i++;
            out.push_back({Tok::Ident, s.substr(st, i - st), st});
        } else if (std::isdigit(c) || (c == '.' && i + 1 < n && std::isdigit((unsigned char)s[i + 1]))) {
            while (i < n && (std::isdigit((unsigned char)s[i]) || s[i] == '.' || s[i] == '_')) i++;
            if (i < n && (s[i] == 'e' || s[i] == 'E')) {
                size_t j = i + 1;
                if (j < n && (s[j] == '+' || s[j] == '-')) j++;
                if (j < n && std::isdigit((unsigned char)s[j])) {
                    i = j;
                    while (i < n && std::isdigit((unsigned char)s[i])) i++;
                }
            }
            // Rust literal suffixes (f64, i32, usize...) are accepted and dropped.
            while (i < n && std::isalnum((unsigned char)s[i])) i++;
            out.push_back({Tok::Number, s.substr(st, i - st), st});
        } else if (c == '=' && i + 1 < n && s[i + 1] == '>') {
            out.push_back({Tok::Punct, "=>", st});
            i += 2;
        } else if (std::strchr(";{},:+@*/()-", c)) {
            out.push_back({Tok::Punct, std::string(1, (char)c), st});
            i++;
        } else {
            return "unexpected character '" + std::string(1, (char)c) + "' at offset " + std::to_string(i);
        }
    }
    out.push_back({Tok::End, "", n});
    return "";
}

struct Parser {
    std::vector<Tok> t;
    size_t k = 0;
    std::map<std::string, int32_t> species, params;
    std::string err;

    const Tok &peek(size_t o = 0) const { return t[std::min(k + o, t.size() - 1)]; }
    bool is(const char *p, size_t o = 0) const { return peek(o).kind == Tok::Punct && peek(o).text == p; }
    bool fail(const std::string &m) {
        if (err.empty()) err = m + " (at offset " + std::to_string(peek().pos) + ")";
        return false;
    }
    bool expect(const char *p) {
        if (!is(p)) return fail(std::string("expected '") + p + "'");
        k++;
        return true;
    }

    static bool parse_number(const std::string &s, double &v) {
        std::string clean;
        for (char c : s) {
            if (c == '_') continue;
            clean.push_back(c);
        }
        // drop a Rust type suffix
        size_t cut = clean.size();
        for (const char *suf : {"f64", "f32", "usize", "isize", "u64", "i64", "u32", "i32"}) {
            size_t L = std::strlen(suf);
            if (clean.size() > L && clean.compare(clean.size() - L, L, suf) == 0) cut = clean.size() - L;
        }
        clean.resize(cut);
        char *end = nullptr;
        v = std::strtod(clean.c_str(), &end);
        return end && *end == '\0' && !clean.empty();
    }

    std::shared_ptr<RateExpr> factor() {
        auto e = std::make_shared<RateExpr>();
        if (is("-")) {
            k++;
            e->op = RateExpr::Neg;
            e->a = factor();
            return e->a ? e : nullptr;
        }
        if (is("(")) {
            k++;
            auto in = expr();
            if (!in || !expect(")")) return nullptr;
            return in;
        }
        const Tok &tk = peek();
        if (tk.kind == Tok::Number) {
            double v;
            if (!parse_number(tk.text, v)) { fail("bad number '" + tk.text + "'"); return nullptr; }
            k++;
            e->op = RateExpr::Const;
            e->value = v;
            return e;
        }
        if (tk.kind == Tok::Ident) {
            auto it = params.find(tk.text);
            if (it == params.end()) {
                if (species.count(tk.text))
                    fail("rate expressions over species are not supported ('" + tk.text + "')");
                else
                    fail("unknown parameter '" + tk.text + "'");
                return nullptr;
            }
            k++;
            e->op = RateExpr::Param;
            e->param = it->second;
            return e;
        }
        fail("expected a rate expression");
        return nullptr;
    }
    std::shared_ptr<RateExpr> term() {
        auto l = factor();
        while (l && (is("*") || is("/"))) {
            auto e = std::make_shared<RateExpr>();
            e->op = is("*") ? RateExpr::Mul : RateExpr::Div;
            k++;
            e->a = l;
            e->b = factor();
            if (!e->b) return nullptr;
            l = e;
        }
        return l;
    }
    std::shared_ptr<RateExpr> expr() {
        auto l = term();
        // A '-' or '+' continues the expression only if the rate does not
        // end here: the next reaction always starts with `ident :`.
        while (l && (is("+") || is("-"))) {
            auto e = std::make_shared<RateExpr>();
            e->op = is("+") ? RateExpr::Add : RateExpr::Sub;
            k++;
            e->a = l;
            e->b = term();
            if (!e->b) return nullptr;
            l = e;
        }
        return l;
    }

    // side := [ [int] ident ( '+' [int] ident )* ]
    bool side(std::vector<Factor> &terms) {
        auto one = [&]() -> bool {
            int32_t mult = 1;
            if (peek().kind == Tok::Number) {
                double v;
                if (!parse_number(peek().text, v) || v != std::floor(v) || v < 1 || v > 1e6)
                    return fail("stoichiometric literal must be a positive integer, got '" + peek().text + "'");
                mult = (int32_t)v;
                k++;
            }
            if (peek().kind != Tok::Ident) return fail("expected a species name");
            auto it = species.find(peek().text);
            if (it == species.end()) return fail("unknown species '" + peek().text + "'");
            terms.push_back({it->second, mult});
            k++;
            return true;
        };
        if (peek().kind == Tok::Ident || peek().kind == Tok::Number) {
            if (!one()) return false;
            while (is("+")) {
                k++;
                if (!one()) return false;
            }
        }
        return true;
    }
};

}  // namespace

std::string parse_dsl(const std::string &text, Network &net) {
    Parser ps;
    std::string terr = tokenize(text, ps.t);
    if (!terr.empty()) return terr;
    // parameters up to ';'
    while (ps.peek().kind == Tok::Ident) {
        const std::string &p = ps.peek().text;
        if (ps.params.count(p)) return "duplicate parameter '" + p + "'";
        ps.params[p] = (int32_t)net.param_names.size();
        net.param_names.push_back(p);
        ps.k++;
    }
    if (!ps.expect(";")) return ps.err;
    if (ps.peek().kind != Tok::Ident) return "expected the system name";
    net.name = ps.peek().text;
    ps.k++;
    if (!ps.expect("{")) return ps.err;
    while (ps.peek().kind == Tok::Ident) {
        const std::string &s = ps.peek().text;
        if (ps.species.count(s) || ps.params.count(s)) return "duplicate name '" + s + "'";
        ps.species[s] = (int32_t)net.species_names.size();
        net.species_names.push_back(s);
        ps.k++;
        if (ps.is(",")) ps.k++;
        else break;
    }
    if (!ps.expect("}")) return ps.err;
    net.n_species = (int32_t)net.species_names.size();
    net.param_values.assign(net.param_names.size(), std::numeric_limits<double>::quiet_NaN());
    net.macro_mode = true;
    while (ps.peek().kind != Tok::End) {
        if (ps.peek().kind != Tok::Ident) return "expected a reaction name";
        Reaction r;
        r.name = ps.peek().text;
        ps.k++;
        if (!ps.expect(":")) return ps.err;
        std::vector<Factor> lhs, rhs;
        if (!ps.side(lhs)) return ps.err;
        if (!ps.expect("=>")) return ps.err;
        if (!ps.side(rhs)) return ps.err;
        if (!ps.expect("@")) return ps.err;
        r.rate_expr = ps.expr();
        if (!r.rate_expr) return ps.err;
        // Propensity factors: each reactant term in the order written
        // (gillespie_macro.rs:106).
        r.factors = lhs;
        // State change: reactants lose their literal, products gain theirs
        // (gillespie_macro.rs:159-163).
        std::vector<int64_t> d(net.n_species, 0);
        for (const Factor &f : lhs) d[f.species] -= f.order;
        for (const Factor &f : rhs) d[f.species] += f.order;
        r.jump = jump_from_dense(d.data(), net.n_species);
        net.reactions.push_back(std::move(r));
    }
    net.refresh_rates();
    return "";
}

}  // namespace rbg
