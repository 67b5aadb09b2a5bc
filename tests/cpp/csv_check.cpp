// Prints what the CSV readers of pansfem2_gb300.hpp make of the files in a directory
// (Node, Element, Dirichlet, Neumann, Periodic, and Initial into nd zeros per node), one
// list per line, numbers with 17 significant digits.  No device call is made.  Built with
// -DVECTOR_ROWS the node rows are a class with the reference's Vector<T> element access
// (operator() and SIZE() only) instead of std::vector<double>.
#include <cstdio>
#include <string>
#include <vector>

#include "pansfem2_gb300.hpp"

using namespace PANSFEM2_GB300;

#ifdef VECTOR_ROWS
class Row {
public:
    Row() {}
    explicit Row(int n) : v_(n, 0.0) {}
    Row(std::vector<double> v) : v_(v) {}
    double &operator()(int i) { return v_[i]; }
    int SIZE() const { return (int)v_.size(); }

private:
    std::vector<double> v_;
};
static double at(Row &r, int i) { return r(i); }
static int len(const Row &r) { return r.SIZE(); }
#else
using Row = std::vector<double>;
static double at(Row &r, int i) { return r[i]; }
static int len(const Row &r) { return (int)r.size(); }
#endif

int main(int argc, char **argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    const int nd = argc > 2 ? std::stoi(argv[2]) : 2;
    std::vector<Row> x;
    std::vector<std::vector<int> > elements;
    std::vector<std::pair<std::pair<int, int>, double> > ufixed, qfixed;
    std::vector<std::pair<int, int> > periodic;
    if (!ImportNodesFromCSV(x, dir + "/Node.csv") || !ImportElementsFromCSV(elements, dir + "/Element.csv") ||
        !ImportDirichletFromCSV(ufixed, dir + "/Dirichlet.csv") || !ImportNeumannFromCSV(qfixed, dir + "/Neumann.csv") ||
        !ImportPeriodicFromCSV(periodic, dir + "/Periodic.csv"))
        return 2;
    std::vector<Row> u(x.size(), Row(nd));
    if (!ImportInitialFromCSV(u, dir + "/Initial.csv")) return 2;
    printf("nodes");
    for (auto &r : x) for (int i = 0; i < len(r); i++) printf(" %.17g", at(r, i));
    printf("\nnode_len");
    for (auto &r : x) printf(" %d", len(r));
    printf("\nconn");
    for (auto &r : elements) for (int v : r) printf(" %d", v);
    printf("\nconn_len");
    for (auto &r : elements) printf(" %d", (int)r.size());
    printf("\nfix");
    for (auto &f : ufixed) printf(" %d %d", f.first.first, f.first.second);
    printf("\nfixval");
    for (auto &f : ufixed) printf(" %.17g", f.second);
    printf("\nload");
    for (auto &f : qfixed) printf(" %d %d", f.first.first, f.first.second);
    printf("\nloadval");
    for (auto &f : qfixed) printf(" %.17g", f.second);
    printf("\nperiodic");
    for (auto &p : periodic) printf(" %d %d", p.first, p.second);
    printf("\ninitial");
    for (auto &r : u) for (int i = 0; i < len(r); i++) printf(" %.17g", at(r, i));
    printf("\n");
    return 0;
}
