/* rebop_gb300.hpp -- the reference's Rust API, in C++, over the C ABI of
 * rebop_gb300.h.
 *
 * `rebop::Gillespie`, `rebop::Rate` and `rebop::Jump` keep the names, argument
 * meanings and order of src/gillespie.rs (Gillespie::new / new_with_seed /
 * seed / add_reaction / get_time / set_time / get_species / set_species /
 * advance_until / _advance_one_reaction, Rate::lma / lma_sparse, Jump::new /
 * new_sparse), so code written against the crate reads the same.  Where the
 * crate panics (assert!, index out of range) these throw std::invalid_argument
 * with the library's message; CUDA failures and timeouts throw
 * std::runtime_error.  `rebop::Ensemble` wraps the batched entry point.
 * Header-only; link -lrebop_gb300. */
#ifndef REBOP_GB300_HPP
#define REBOP_GB300_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "rebop_gb300.h"

namespace rebop {

namespace detail {
inline std::string last_error() {
    char buf[1024];
    rb_last_error(buf, sizeof buf);
    return buf;
}
inline void check(int status) {
    if (status == RB_OK) return;
    if (status == RB_ERR_INVALID || status == RB_ERR_PARSE) throw std::invalid_argument(last_error());
    throw std::runtime_error(last_error());
}
}  // namespace detail

/* Rate::LMA / Rate::LMASparse (gillespie.rs:12-35). */
class Rate {
public:
    /* Rate::lma(rate, reactants): one exponent per species. */
    static Rate lma(double rate, std::vector<uint32_t> exponents) {
        Rate r;
        r.rate_ = rate;
        r.dense_ = std::move(exponents);
        return r;
    }
    /* Rate::lma_sparse(rate, [(species, exponent), ...]), multiplied in the order given. */
    static Rate lma_sparse(double rate, std::vector<std::pair<uint32_t, uint32_t>> pairs) {
        Rate r;
        r.rate_ = rate;
        r.sparse_ = true;
        r.pairs_ = std::move(pairs);
        return r;
    }
    double rate() const { return rate_; }
    bool is_sparse() const { return sparse_; }
    const std::vector<uint32_t> &exponents() const { return dense_; }
    const std::vector<std::pair<uint32_t, uint32_t>> &pairs() const { return pairs_; }

private:
    double rate_ = 0.0;
    bool sparse_ = false;
    std::vector<uint32_t> dense_;
    std::vector<std::pair<uint32_t, uint32_t>> pairs_;
};

/* Jump::new / Jump::new_sparse (gillespie.rs:95-152): the net change per species. */
class Jump {
public:
    static Jump new_dense(std::vector<int64_t> differences) {
        Jump j;
        j.d_ = std::move(differences);
        return j;
    }
    /* (species, difference) pairs over n_species species. */
    static Jump new_sparse(const std::vector<std::pair<uint32_t, int64_t>> &pairs, size_t n_species) {
        Jump j;
        j.d_.assign(n_species, 0);
        for (const auto &p : pairs) {
            if (p.first >= n_species) throw std::invalid_argument("jump species index out of range");
            j.d_[p.first] += p.second;
        }
        return j;
    }
    const std::vector<int64_t> &differences() const { return d_; }

private:
    std::vector<int64_t> d_;
};

/* The Rust crate's `Gillespie` (gillespie.rs:157-344): one trajectory whose
 * every advance runs on the GPU. */
class Gillespie {
public:
    /* Gillespie::new(species, sparse): seeded from OS entropy. */
    Gillespie(const std::vector<int64_t> &species, bool sparse) {
        detail::check(rb_gillespie_new(species.data(), (int32_t)species.size(), sparse ? 1 : 0, &g_));
    }
    /* Gillespie::new_with_seed(species, sparse, seed). */
    static Gillespie new_with_seed(const std::vector<int64_t> &species, bool sparse, uint64_t seed) {
        rb_gillespie *g = nullptr;
        detail::check(rb_gillespie_new_with_seed(species.data(), (int32_t)species.size(), sparse ? 1 : 0, seed, &g));
        return Gillespie(g);
    }
    Gillespie(const Gillespie &) = delete;
    Gillespie &operator=(const Gillespie &) = delete;
    Gillespie(Gillespie &&o) noexcept : g_(o.g_) { o.g_ = nullptr; }
    Gillespie &operator=(Gillespie &&o) noexcept {
        if (this != &o) {
            if (g_) rb_gillespie_free(g_);
            g_ = o.g_;
            o.g_ = nullptr;
        }
        return *this;
    }
    ~Gillespie() {
        if (g_) rb_gillespie_free(g_);
    }

    void seed(uint64_t seed) { detail::check(rb_gillespie_seed(g_, seed)); }
    size_t nb_species() const { return (size_t)rb_gillespie_nb_species(g_); }
    size_t nb_reactions() const { return (size_t)rb_gillespie_nb_reactions(g_); }

    /* add_reaction(rate, differences): both sized to the species count, or
     * std::invalid_argument as the crate's assert_eq! panics. */
    void add_reaction(const Rate &rate, const Jump &jump) { add_reaction(rate, jump.differences()); }
    void add_reaction(const Rate &rate, const std::vector<int64_t> &differences) {
        if (rate.is_sparse()) {
            std::vector<uint32_t> sp, ex;
            for (const auto &p : rate.pairs()) {
                sp.push_back(p.first);
                ex.push_back(p.second);
            }
            detail::check(rb_gillespie_add_reaction_lma_sparse(g_, rate.rate(), sp.data(), ex.data(),
                                                               (int32_t)sp.size(), differences.data(),
                                                               (int32_t)differences.size()));
        } else {
            detail::check(rb_gillespie_add_reaction_lma(g_, rate.rate(), rate.exponents().data(),
                                                        (int32_t)rate.exponents().size(), differences.data(),
                                                        (int32_t)differences.size()));
        }
    }

    double get_time() const { return rb_gillespie_get_time(g_); }
    void set_time(double t) { rb_gillespie_set_time(g_, t); }
    int64_t get_species(size_t s) const {
        int64_t v = 0;
        detail::check(rb_gillespie_get_species(g_, (int32_t)s, &v));
        return v;
    }
    void set_species(const std::vector<int64_t> &species) {
        detail::check(rb_gillespie_set_species(g_, species.data(), (int32_t)species.size()));
    }
    /* advance_until(tmax) (gillespie.rs:315-344). */
    void advance_until(double tmax) { detail::check(rb_gillespie_advance_until(g_, tmax)); }
    /* _advance_one_reaction (gillespie.rs:275-297). */
    void advance_one_reaction() { detail::check(rb_gillespie_advance_one_reaction(g_)); }

private:
    explicit Gillespie(rb_gillespie *g) : g_(g) {}
    rb_gillespie *g_ = nullptr;
};

/* Many independent trajectories of one network in one launch
 * (rb_ensemble_run): counts[i][s][j] is species save[s] of trajectory j at
 * the i-th of nb_steps + 1 sample times tmax * i / nb_steps. */
class Ensemble {
public:
    explicit Ensemble(size_t n_species) { detail::check(rb_network_create((int32_t)n_species, &net_)); }
    /* A define_system! body (src/gillespie_macro.rs:50-58), with the macro's
     * arithmetic; its parameters start as NaN (set_param). */
    static Ensemble from_dsl(const std::string &text) {
        rb_network *n = nullptr;
        detail::check(rb_network_from_dsl(text.c_str(), &n));
        return Ensemble(n);
    }
    Ensemble(const Ensemble &) = delete;
    Ensemble &operator=(const Ensemble &) = delete;
    Ensemble(Ensemble &&o) noexcept : net_(o.net_) { o.net_ = nullptr; }
    ~Ensemble() {
        if (net_) rb_network_destroy(net_);
    }
    void set_param(const std::string &name, double value) {
        detail::check(rb_network_set_param(net_, name.c_str(), value));
    }
    std::vector<std::string> params() const { return names(rb_network_nb_params(net_), rb_network_param_name); }
    std::vector<std::string> species() const {
        return names(rb_network_nb_species(net_), rb_network_species_name);
    }
    double reaction_rate(size_t r) const {
        double v = 0.0;
        detail::check(rb_network_reaction_rate(net_, (int32_t)r, &v));
        return v;
    }
    size_t nb_species() const { return (size_t)rb_network_nb_species(net_); }
    size_t nb_reactions() const { return (size_t)rb_network_nb_reactions(net_); }
    void add_reaction(const Rate &rate, const std::vector<int64_t> &differences) {
        if (rate.is_sparse()) {
            std::vector<uint32_t> sp, ex;
            for (const auto &p : rate.pairs()) {
                sp.push_back(p.first);
                ex.push_back(p.second);
            }
            detail::check(rb_network_add_reaction_lma_sparse(net_, rate.rate(), sp.data(), ex.data(),
                                                             (int32_t)sp.size(), differences.data(),
                                                             (int32_t)differences.size()));
        } else {
            detail::check(rb_network_add_reaction_lma(net_, rate.rate(), rate.exponents().data(),
                                                      (int32_t)rate.exponents().size(), differences.data(),
                                                      (int32_t)differences.size()));
        }
    }
    struct Result {
        std::vector<int64_t> counts;  /* [nb_steps + 1][n_saved][n_traj] */
        std::vector<double> times;    /* [nb_steps + 1] */
        std::vector<uint64_t> events; /* [n_traj] */
        rb_run_stats stats{};
    };
    /* One trajectory per seed from the shared initial counts x0; every
     * species is saved. */
    Result run(const std::vector<int64_t> &x0, const std::vector<uint64_t> &seeds, double tmax,
               int64_t nb_steps) const {
        Result r;
        const size_t n = seeds.size(), S = nb_species();
        if (x0.size() != S)
            throw std::invalid_argument("x0 has " + std::to_string(x0.size()) + " counts for " +
                                        std::to_string(S) + " species");
        if (nb_steps < 1) throw std::invalid_argument("nb_steps must be >= 1");
        r.counts.resize((size_t)(nb_steps + 1) * S * n);
        r.times.resize((size_t)nb_steps + 1);
        r.events.resize(n);
        detail::check(rb_ensemble_run(net_, (int64_t)n, x0.data(), 0, nullptr, 0, seeds.data(), tmax, nb_steps,
                                      nullptr, -1, r.counts.data(), r.times.data(), r.events.data(), nullptr,
                                      &r.stats));
        return r;
    }

private:
    explicit Ensemble(rb_network *n) : net_(n) {}
    std::vector<std::string> names(int32_t n, int (*get)(const rb_network *, int32_t, char *, size_t)) const {
        std::vector<std::string> out;
        char buf[256];
        for (int32_t i = 0; i < n; ++i) {
            detail::check(get(net_, i, buf, sizeof buf));
            out.emplace_back(buf);
        }
        return out;
    }
    rb_network *net_ = nullptr;
};

}  // namespace rebop

#endif /* REBOP_GB300_HPP */
