// params_from / growth_from / generations_from on a stand-in for boost::property_tree::ptree: a tree of
// (key, child) pairs with string data, dotted paths, get<T>(path, default), get_child_optional and
// get_child.  Exits non-zero on the first mismatch.
#include <cstdio>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "clotho_gb300/cpp/clotho_gb300.hpp"

struct Tree {
    std::string value;
    std::vector<std::pair<std::string, Tree>> kids;

    const std::string& data() const { return value; }
    auto begin() const { return kids.begin(); }
    auto end() const { return kids.end(); }

    const Tree* find(const std::string& path) const {
        const Tree* t = this;
        std::string rest = path;
        while (!rest.empty()) {
            const size_t dot = rest.find('.');
            const std::string head = rest.substr(0, dot);
            rest = dot == std::string::npos ? "" : rest.substr(dot + 1);
            const Tree* next = nullptr;
            for (const auto& kv : t->kids)
                if (kv.first == head) { next = &kv.second; break; }
            if (!next) return nullptr;
            t = next;
        }
        return t;
    }
    const Tree* get_child_optional(const std::string& path) const { return find(path); }
    const Tree& get_child(const std::string& path) const { return *find(path); }
    template <class T>
    T get(const std::string& path, const T& dflt) const {
        const Tree* t = find(path);
        if (!t) return dflt;
        std::istringstream in(t->value);
        T v{};
        in >> v;
        return v;
    }
    Tree& put(const std::string& key, const std::string& v) {
        kids.push_back({key, Tree{v, {}}});
        return kids.back().second;
    }
    Tree& child(const std::string& key) {
        kids.push_back({key, Tree{}});
        return kids.back().second;
    }
};
template <>
std::string Tree::get<std::string>(const std::string& path, const std::string& dflt) const {
    const Tree* t = find(path);
    return t ? t->value : dflt;
}

static int fails = 0;
#define CHECK(c)                                                        \
    do {                                                                \
        if (!(c)) { std::printf("FAILED: %s (line %d)\n", #c, __LINE__); ++fails; } \
    } while (0)

int main() {
    using namespace clotho::gb300;
    Tree empty;
    Parameters d = params_from(empty, 500, 4096);
    CHECK(d.mu == 1e-4 && d.rho == 1e-4 && d.bias == 0.5 && d.traits == 1 && d.p_neutral == 0.5);
    CHECK(d.eff_mean == 0.0 && d.eff_sigma == 1.0 && d.fitness == CLOTHO_FIT_CONSTANT && d.seed == 0);
    CHECK(d.max_individuals == 500 && d.max_alleles == 4096);
    CHECK(!growth_from(empty) && generations_from(empty) == 10000u);

    Tree root;
    Tree& c = root.child("configuration");
    c.child("generations").put("size", "25");
    Tree& g = c.child("population_growth");
    g.put("name", "predefined");
    Tree& sizes = g.child("params").child("sizes");
    sizes.put("", "100");
    sizes.put("", "40");
    c.child("mutation").put("mu", "0.01");
    Tree& rec = c.child("recombination");
    rec.put("rho", "0.5");
    rec.child("sequence_bias").put("p", "0.3");
    Tree& tr = c.child("traits");
    tr.put("N", "2");
    tr.put("mean", "0.1");
    tr.put("sigma", "2");
    c.child("neutral").put("p", "0.2");
    Tree& f = c.child("fitness");
    f.put("name", "quadratic");
    f.child("params").put("scale", "3");
    c.child("random_number").put("seed", "42");

    Parameters p = params_from(root, 100, 8192);
    CHECK(p.mu == 0.01 && p.rho == 0.5 && p.bias == 0.3 && p.traits == 2 && p.p_neutral == 0.2);
    CHECK(p.eff_mean == 0.1 && p.eff_sigma == 2.0 && p.fitness == CLOTHO_FIT_QUADRATIC && p.fit_param == 3.0);
    CHECK(p.seed == 42 && generations_from(root) == 25u);
    auto gr = growth_from(root);
    CHECK(gr && (*gr)(0u, 0u) == 100u && (*gr)(100u, 1u) == 40u && (*gr)(40u, 2u) == 100u);

    Tree lin;
    Tree& lg = lin.child("population_growth");
    lg.put("name", "linear");
    Tree& lp = lg.child("params");
    lp.put("A", "1.5");
    lp.put("B", "10");
    auto lgr = growth_from(lin);   // no "configuration" block: the root is the configuration
    CHECK(lgr && (*lgr)(0u, 0u) == 10u && (*lgr)(10u, 1u) == 25u);

    Tree bad;
    bad.child("fitness").put("name", "random");
    bool threw = false;
    try { params_from(bad, 1, 64); } catch (const Error&) { threw = true; }
    CHECK(threw);
    if (fails == 0) std::printf("ok\n");
    return fails == 0 ? 0 : 1;
}
