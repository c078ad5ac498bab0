// ref_passive_harness.cpp -- drives the reference's own HinesMatrix and
// HSolvePassive classes (hsolve/HinesMatrix.cpp, hsolve/HSolvePassive.cpp)
// on trees given in Hines order, the way the reference's unit tests
// testHinesMatrix / testHSolvePassive do (hsolve/HinesMatrix.cpp:478-755,
// hsolve/HSolvePassive.cpp:452-987), and prints every intermediate value as a
// hex float so that golden vectors carry the reference's exact bits.
//
// Test infrastructure: built by oracle/build_ref.py into oracle/_ref/ and run
// only by tests/golden/make_golden.py in a container that has the reference.
//
// stdin, one cell per record:
//   n dt
//   for each compartment i: nchildren child...
//   Ra[n] Rm[n] Cm[n] Em[n] V[n]     (hex or decimal doubles)
// stdout, per cell: "A0" dense matrix after setup, then for each of 2 passes
//   "B" after updateMatrix, "FA"/"FB" after forwardEliminate,
//   "VMID"/"V" after backwardSubstitute.
#include "HSolvePassive.h"

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

class PassiveHarness : public HSolvePassive {
public:
    void build(const std::vector<TreeNodeStruct>& tree, const std::vector<double>& Em,
               const std::vector<double>& V, double dt) {
        tree_ = tree;
        V_ = V;
        compartment_.clear();
        for (size_t i = 0; i < tree.size(); ++i) {
            CompartmentStruct c;
            c.CmByDt = 2.0 * tree[i].Cm / dt;
            c.EmByRm = Em[i] / tree[i].Rm;
            compartment_.push_back(c);
        }
        HinesMatrix::setup(tree_, dt);
    }
    void update() { updateMatrix(); }
    void forward() { forwardEliminate(); }
    void backward() { backwardSubstitute(); }
    double v(unsigned i) const { return V_[i]; }
};

static void dumpA(const char* tag, const PassiveHarness& h, unsigned n) {
    std::printf("%s", tag);
    for (unsigned i = 0; i < n; ++i)
        for (unsigned j = 0; j < n; ++j) std::printf(" %a", h.getA(i, j));
    std::printf("\n");
}
template <class F>
static void dumpVec(const char* tag, unsigned n, F f) {
    std::printf("%s", tag);
    for (unsigned i = 0; i < n; ++i) std::printf(" %a", f(i));
    std::printf("\n");
}

static double readD() {
    std::string s;
    std::cin >> s;
    return std::strtod(s.c_str(), nullptr);
}

int main() {
    unsigned n;
    while (std::cin >> n) {
        double dt = readD();
        std::vector<TreeNodeStruct> tree(n);
        for (unsigned i = 0; i < n; ++i) {
            unsigned k;
            std::cin >> k;
            for (unsigned j = 0; j < k; ++j) {
                unsigned c;
                std::cin >> c;
                tree[i].children.push_back(c);
            }
        }
        std::vector<double> Em(n), V(n);
        for (unsigned i = 0; i < n; ++i) tree[i].Ra = readD();
        for (unsigned i = 0; i < n; ++i) tree[i].Rm = readD();
        for (unsigned i = 0; i < n; ++i) tree[i].Cm = readD();
        for (unsigned i = 0; i < n; ++i) Em[i] = readD();
        for (unsigned i = 0; i < n; ++i) V[i] = readD();
        PassiveHarness h;
        h.build(tree, Em, V, dt);
        std::printf("CELL %u\n", n);
        dumpA("A0", h, n);
        for (int pass = 0; pass < 2; ++pass) {
            h.update();
            dumpVec("B", n, [&](unsigned i) { return h.getB(i); });
            h.forward();
            dumpA("FA", h, n);
            dumpVec("FB", n, [&](unsigned i) { return h.getB(i); });
            h.backward();
            dumpVec("VMID", n, [&](unsigned i) { return h.getVMid(i); });
            dumpVec("V", n, [&](unsigned i) { return h.v(i); });
        }
        std::fflush(stdout);
    }
    return 0;
}
