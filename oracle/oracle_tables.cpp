// Oracle polynomial evaluators (test infrastructure; see oracle.h).
//
// The MB-pol 2B/3B energies are E(x) = sum_k a[k] * P_k(x) where P_k is the sum
// of the monomials of one permutation orbit (SOURCE/poly-2b-v6x.cpp:5,
// SOURCE/poly-3b-v2x.cpp:5 evaluate the same polynomials in a generated nested
// form).  Two evaluators live here:
//   * naive: every monomial multiplied out, gradient by the product rule;
//   * trie:  the monomials arranged as a prefix tree over sorted variable
//            indices and walked depth first, carrying prefix products (the
//            adjoints) down and subtree sums up, so value and gradient cost
//            about two multiply-adds per monomial.
#include "oracle.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

struct PolyTable {
    int n_vars = 0;
    std::vector<double> coef;                 // a[k]
    std::vector<int> mono_k;                  // coefficient index per monomial
    std::vector<std::vector<int>> mono_v;     // sorted variable indices
    // depth-first program
    std::vector<int> op;    // 0 = enter(var), 1 = leaf(var, coef), 2 = exit(var)
    std::vector<int> var;
    std::vector<double> c;  // leaf coefficient, or the node's own coefficient on enter
    double root_c = 0.0;
    bool loaded = false;
};

PolyTable g_t2, g_t3;

struct TrieNode {
    std::map<int, TrieNode*> ch;
    bool has_c = false;
    double c = 0.0;
    ~TrieNode() { for (auto& kv : ch) delete kv.second; }
};

void build_program(PolyTable& t) {
    TrieNode root;
    for (size_t m = 0; m < t.mono_v.size(); ++m) {
        TrieNode* n = &root;
        for (int v : t.mono_v[m]) {
            auto it = n->ch.find(v);
            if (it == n->ch.end()) it = n->ch.emplace(v, new TrieNode).first;
            n = it->second;
        }
        n->has_c = true;
        n->c = t.coef[t.mono_k[m]];
    }
    t.root_c = root.has_c ? root.c : 0.0;
    struct Frame { TrieNode* n; std::map<int, TrieNode*>::iterator it; int var; };
    std::vector<Frame> st;
    st.push_back({&root, root.ch.begin(), -1});
    while (!st.empty()) {
        Frame& f = st.back();
        if (f.it == f.n->ch.end()) {
            if (f.var >= 0) { t.op.push_back(2); t.var.push_back(f.var); t.c.push_back(0.0); }
            st.pop_back();
            continue;
        }
        int v = f.it->first;
        TrieNode* child = f.it->second;
        ++f.it;
        if (child->ch.empty()) {
            t.op.push_back(1); t.var.push_back(v); t.c.push_back(child->c);
        } else {
            t.op.push_back(0); t.var.push_back(v); t.c.push_back(child->has_c ? child->c : 0.0);
            st.push_back({child, child->ch.begin(), v});
        }
    }
}

int load_one(const char* path, int n_vars, PolyTable& t) {
    FILE* fp = std::fopen(path, "r");
    if (!fp) return 1;
    t = PolyTable();
    t.n_vars = n_vars;
    char line[512];
    while (std::fgets(line, sizeof line, fp)) {
        if (line[0] == 'C') {
            int k; double a;
            if (std::sscanf(line + 1, "%d %lf", &k, &a) != 2) { std::fclose(fp); return 2; }
            if ((int)t.coef.size() != k) { std::fclose(fp); return 3; }
            t.coef.push_back(a);
        } else if (line[0] == 'M') {
            char* p = line + 1;
            char* end;
            int k = (int)std::strtol(p, &end, 10);
            std::vector<int> vs;
            p = end;
            while (true) {
                long v = std::strtol(p, &end, 10);
                if (end == p) break;
                if (v < 0 || v >= n_vars) { std::fclose(fp); return 4; }
                vs.push_back((int)v);
                p = end;
            }
            t.mono_k.push_back(k);
            t.mono_v.push_back(vs);
        }
    }
    std::fclose(fp);
    build_program(t);
    t.loaded = true;
    return 0;
}

double eval_trie(const PolyTable& t, const double* x, double* g) {
    for (int j = 0; j < t.n_vars; ++j) g[j] = 0.0;
    double pi[8], S[8];
    int d = 0;
    pi[0] = 1.0;
    S[0] = t.root_c;
    const size_t n = t.op.size();
    for (size_t i = 0; i < n; ++i) {
        const int v = t.var[i];
        switch (t.op[i]) {
        case 0:  // enter child v
            pi[d + 1] = pi[d] * x[v];
            S[d + 1] = t.c[i];
            ++d;
            break;
        case 1:  // leaf child v with coefficient c
            S[d] += x[v] * t.c[i];
            g[v] += pi[d] * t.c[i];
            break;
        default:  // leave child v
            S[d - 1] += x[v] * S[d];
            g[v] += pi[d - 1] * S[d];
            --d;
            break;
        }
    }
    return S[0];
}

double eval_naive(const PolyTable& t, const double* x, double* g) {
    for (int j = 0; j < t.n_vars; ++j) g[j] = 0.0;
    double e = 0.0;
    for (size_t m = 0; m < t.mono_v.size(); ++m) {
        const std::vector<int>& vs = t.mono_v[m];
        const double a = t.coef[t.mono_k[m]];
        double prod = a;
        for (int v : vs) prod *= x[v];
        e += prod;
        for (size_t p = 0; p < vs.size(); ++p) {
            double d = a;
            for (size_t q = 0; q < vs.size(); ++q)
                if (q != p) d *= x[vs[q]];
            g[vs[p]] += d;
        }
    }
    return e;
}

}  // namespace

extern "C" int orc_load_tables(const char* p2, const char* p3) {
    int rc = load_one(p2, 31, g_t2);
    if (rc) return 10 + rc;
    rc = load_one(p3, 36, g_t3);
    if (rc) return 20 + rc;
    if (g_t2.coef.size() != 1153 || g_t3.coef.size() != 1163) return 30;
    return 0;
}

static void require(const PolyTable& t) {
    if (!t.loaded) {
        std::fprintf(stderr, "oracle: polynomial tables not loaded (call orc_load_tables)\n");
        std::abort();
    }
}

extern "C" double orc_poly2b(const double x[31], double g[31]) { require(g_t2); return eval_trie(g_t2, x, g); }
extern "C" double orc_poly3b(const double x[36], double g[36]) { require(g_t3); return eval_trie(g_t3, x, g); }
extern "C" double orc_poly2b_naive(const double x[31], double g[31]) { require(g_t2); return eval_naive(g_t2, x, g); }
extern "C" double orc_poly3b_naive(const double x[36], double g[36]) { require(g_t3); return eval_naive(g_t3, x, g); }
