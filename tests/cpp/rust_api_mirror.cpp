// The C++ mirror of the crate's API (include/rebop_gb300.hpp), exercised the
// way tests in src/gillespie.rs use the Rust one.  Argument "cpu": only the
// calls that need no GPU; "gpu": also advance a dimer trajectory and run an
// ensemble, printing the results for the test to compare with the oracle.
#include <cstdio>
#include <cstring>
#include <stdexcept>

#include "rebop_gb300.hpp"

static int fails = 0;
#define EXPECT(c)                                                      \
    do {                                                               \
        if (!(c)) {                                                    \
            std::fprintf(stderr, "line %d: %s\n", __LINE__, #c);       \
            ++fails;                                                   \
        }                                                              \
    } while (0)

static void add_dimer(rebop::Gillespie &g) {
    g.add_reaction(rebop::Rate::lma(25.0, {1, 0, 0, 0}), std::vector<int64_t>{0, 1, 0, 0});
    g.add_reaction(rebop::Rate::lma(1000.0, {0, 1, 0, 0}), rebop::Jump::new_dense({0, 0, 1, 0}));
    g.add_reaction(rebop::Rate::lma(0.001, {0, 0, 2, 0}), rebop::Jump::new_sparse({{2, -2}, {3, 1}}, 4));
    g.add_reaction(rebop::Rate::lma_sparse(0.1, {{1, 1}}), std::vector<int64_t>{0, -1, 0, 0});
    g.add_reaction(rebop::Rate::lma(1.0, {0, 0, 1, 0}), std::vector<int64_t>{0, 0, -1, 0});
}

int main(int argc, char **argv) {
    const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
    auto g = rebop::Gillespie::new_with_seed({1, 0, 0, 0}, false, 777);
    add_dimer(g);
    EXPECT(g.nb_species() == 4 && g.nb_reactions() == 5);
    EXPECT(g.get_time() == 0.0 && g.get_species(0) == 1 && g.get_species(3) == 0);
    // assert_eq! on the vector lengths (gillespie.rs:227-237) throws
    bool threw = false;
    try {
        g.add_reaction(rebop::Rate::lma(1.0, {1, 0}), std::vector<int64_t>{0, 0, 0, 0});
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    EXPECT(threw && g.nb_reactions() == 5);
    threw = false;
    try {  // issue 85: sparse index out of range (gillespie.rs:496-502)
        g.add_reaction(rebop::Rate::lma_sparse(1.0, {{10, 1}}), std::vector<int64_t>{0, 0, 0, 0});
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    EXPECT(threw);
    threw = false;
    try {
        g.get_species(4);
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    EXPECT(threw);
    rebop::Ensemble e(4);
    e.add_reaction(rebop::Rate::lma(25.0, {1, 0, 0, 0}), {0, 1, 0, 0});
    e.add_reaction(rebop::Rate::lma(1000.0, {0, 1, 0, 0}), {0, 0, 1, 0});
    e.add_reaction(rebop::Rate::lma(0.001, {0, 0, 2, 0}), {0, 0, -2, 1});
    e.add_reaction(rebop::Rate::lma(0.1, {0, 1, 0, 0}), {0, -1, 0, 0});
    e.add_reaction(rebop::Rate::lma(1.0, {0, 0, 1, 0}), {0, 0, -1, 0});
    EXPECT(e.nb_species() == 4 && e.nb_reactions() == 5);
    // Ensemble::run checks its arguments before any GPU work
    threw = false;
    try {
        e.run({1, 0, 0}, {1, 2}, 1.0, 10);  // 3 counts for 4 species
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    EXPECT(threw);
    threw = false;
    try {
        e.run({1, 0, 0, 0}, {1, 2}, 1.0, -5);
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    EXPECT(threw);
    // define_system! (gillespie_macro.rs:50-58): parameters start NaN
    auto d = rebop::Ensemble::from_dsl(
        "rtx rtl rdi rdm rdp; Dimers { gene, mRNA, protein, dimer } "
        "transcription: gene => gene + mRNA @ rtx translation: mRNA => mRNA + protein @ rtl "
        "dimerization: 2 protein => dimer @ rdi decay_mRNA: mRNA => @ rdm decay_prot: protein => @ rdp");
    EXPECT(d.nb_species() == 4 && d.nb_reactions() == 5 && d.params().size() == 5);
    EXPECT(d.species()[2] == "protein" && d.params()[1] == "rtl");
    EXPECT(d.reaction_rate(1) != d.reaction_rate(1));  // NaN
    d.set_param("rtl", 1000.0);
    EXPECT(d.reaction_rate(1) == 1000.0);
    threw = false;
    try {
        rebop::Ensemble::from_dsl("k; X { A } r: B => A @ k");
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    EXPECT(threw);
    if (gpu) {
        for (double tm : {0.1, 0.25, 0.7}) g.advance_until(tm);
        std::printf("traj %.17g %lld %lld %lld %lld\n", g.get_time(), (long long)g.get_species(0),
                    (long long)g.get_species(1), (long long)g.get_species(2), (long long)g.get_species(3));
        std::vector<uint64_t> seeds;
        for (uint64_t s = 1; s <= 64; ++s) seeds.push_back(s * 0x9E3779B97F4A7C15ull);
        const auto r = e.run({1, 0, 0, 0}, seeds, 0.5, 5);
        unsigned long long total = 0;
        for (uint64_t v : r.events) total += v;
        std::printf("ensemble %llu", total);
        for (size_t j = 0; j < seeds.size(); ++j) std::printf(" %lld", (long long)r.counts[(5 * 4 + 3) * 64 + j]);
        std::printf("\n");
    }
    std::printf(fails ? "FAILED %d\n" : "ok\n", fails);
    return fails ? 1 : 0;
}
