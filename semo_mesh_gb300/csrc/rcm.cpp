// Reverse Cuthill-McKee ordering of the cell graph, host side.
//
// SEMO orders cells with SPARSEPAK's GENRCM (George & Liu, "Computer Solution
// of Large Sparse Positive Definite Systems", 1981), through
// SEMO_Utility_Math::lib_RCM (src/math/RCM.cpp:34-218; genrcm :1214,
// root_find :3585, level_set :2541, degree :1075, rcm :3353).  The result
// depends on every tie-break, so this is the same published algorithm, step
// for step:
//   * components are started from the lowest-numbered unvisited node;
//   * a pseudo-peripheral root is found by repeated level structures, taking
//     the first node of minimum degree in the last level;
//   * Cuthill-McKee numbers each node's unvisited neighbours in adjacency
//     order, then stably sorts that run by ascending degree (degree counted
//     inside the component);
//   * each component's order is reversed.
// Adjacency lists are 1-based, in the order SEMO builds them: each cell's
// internal faces in ascending face order.
#include <cstdlib>
#include <vector>

#include "semo_internal.h"

namespace {

struct Graph {
    const int* xadj;  // 1-based offsets, size n+1
    const int* adj;   // 1-based node ids
};

// Level structure rooted at `root` over nodes with mask != 0 (masks are
// restored on exit).  Returns the number of levels; ls holds the nodes,
// xls the 1-based level starts.
int level_structure(const Graph& g, int root, int* mask, int* xls, int* ls) {
    mask[root - 1] = 0;
    ls[0] = root;
    int nlvl = 0, lvlend = 0, size = 1;
    for (;;) {
        int lbegin = lvlend + 1;
        lvlend = size;
        xls[nlvl++] = lbegin;
        for (int i = lbegin; i <= lvlend; ++i) {
            int node = ls[i - 1];
            for (int j = g.xadj[node - 1]; j < g.xadj[node]; ++j) {
                int nb = g.adj[j - 1];
                if (mask[nb - 1]) { ls[size++] = nb; mask[nb - 1] = 0; }
            }
        }
        if (size - lvlend <= 0) break;
    }
    xls[nlvl] = lvlend + 1;
    for (int i = 0; i < size; ++i) mask[ls[i] - 1] = 1;
    return nlvl;
}

int pseudo_peripheral(const Graph& g, int root, int* mask, int* xls, int* ls) {
    int nlvl = level_structure(g, root, mask, xls, ls);
    int size = xls[nlvl] - 1;
    if (nlvl == 1 || nlvl == size) return root;
    for (;;) {
        int mindeg = size, first = xls[nlvl - 1];
        root = ls[first - 1];
        if (first < size) {
            for (int j = first; j <= size; ++j) {
                int node = ls[j - 1], deg = 0;
                for (int k = g.xadj[node - 1]; k < g.xadj[node]; ++k)
                    if (mask[g.adj[k - 1] - 1] > 0) ++deg;
                if (deg < mindeg) { root = node; mindeg = deg; }
            }
        }
        int nlvl2 = level_structure(g, root, mask, xls, ls);
        if (nlvl2 <= nlvl) break;
        nlvl = nlvl2;
        if (size <= nlvl) break;
    }
    return root;
}

// Degrees inside the component of `root`; the sign of xadj marks visited
// nodes temporarily, as in SPARSEPAK's DEGREE.
int component_degrees(const Graph& g, int* xadj_mut, int root, const int* mask, int* deg, int* ls) {
    ls[0] = root;
    xadj_mut[root - 1] = -xadj_mut[root - 1];
    int lvlend = 0, size = 1;
    for (;;) {
        int lbegin = lvlend + 1;
        lvlend = size;
        for (int i = lbegin; i <= lvlend; ++i) {
            int node = ls[i - 1];
            int jb = -xadj_mut[node - 1], je = std::abs(xadj_mut[node]) - 1, d = 0;
            for (int j = jb; j <= je; ++j) {
                int nb = g.adj[j - 1];
                if (mask[nb - 1]) {
                    ++d;
                    if (xadj_mut[nb - 1] >= 0) { xadj_mut[nb - 1] = -xadj_mut[nb - 1]; ls[size++] = nb; }
                }
            }
            deg[node - 1] = d;
        }
        if (size - lvlend == 0) break;
    }
    for (int i = 0; i < size; ++i) xadj_mut[ls[i] - 1] = -xadj_mut[ls[i] - 1];
    return size;
}

int cuthill_mckee(const Graph& g, int* xadj_mut, int root, int* mask, int* perm, int* deg) {
    int size = component_degrees(g, xadj_mut, root, mask, deg, perm);
    mask[root - 1] = 0;
    if (size == 1) return 1;
    int lvlend = 0, lnbr = 1;
    while (lvlend < lnbr) {
        int lbegin = lvlend + 1;
        lvlend = lnbr;
        for (int i = lbegin; i <= lvlend; ++i) {
            int node = perm[i - 1];
            int fnbr = lnbr + 1;
            for (int j = g.xadj[node - 1]; j < g.xadj[node]; ++j) {
                int nb = g.adj[j - 1];
                if (mask[nb - 1]) { mask[nb - 1] = 0; perm[lnbr++] = nb; }
            }
            if (lnbr <= fnbr) continue;
            // stable insertion sort of the new run perm[fnbr-1 .. lnbr-1] by degree
            for (int k = fnbr; k < lnbr; ++k) {
                int nb = perm[k];
                int l = k;
                while (l > fnbr) {
                    int prev = perm[l - 1];
                    if (deg[prev - 1] <= deg[nb - 1]) break;
                    perm[l] = prev;
                    --l;
                }
                perm[l] = nb;
            }
        }
    }
    for (int a = 0, b = size - 1; a < b; ++a, --b) std::swap(perm[a], perm[b]);
    return size;
}

}  // namespace

namespace semo {

// perm[r] (0-based) = node placed at position r.
void genrcm_perm(int n, const std::vector<int>& xadj, const std::vector<int>& adj, std::vector<int>& perm) {
    std::vector<int> xm(xadj.begin(), xadj.end());
    Graph g{xadj.data(), adj.data()};
    std::vector<int> mask(n, 1), xls(n + 1), p1(n), deg(n);
    int num = 1;
    for (int i = 0; i < n; ++i) {
        if (!mask[i]) continue;
        int root = pseudo_peripheral(g, i + 1, mask.data(), xls.data(), p1.data() + num - 1);
        num += cuthill_mckee(g, xm.data(), root, mask.data(), p1.data() + num - 1, deg.data());
        if (num > n) break;
    }
    perm.resize(n);
    for (int i = 0; i < n; ++i) perm[i] = p1[i] - 1;
}

}  // namespace semo
