// peelone_dyn: drop-in for the reference's peel/main.cu binary (Makefile target
// peelone_dyn): loads the graph with the de-duplicating CSR loader, prints V,
// E, the degree standard deviation and the maximum degree, then times
// peel_dyn and peelone_dyn ten times each (repSimulation, main.cu:28-49:
// the minimum and maximum are dropped from the average) and prints Kmax.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "_common.h"

static int method_run(kc_graph *g, int method, uint32_t *kmax) {
    kc_stats st;
    if (kc_decompose(g, method, nullptr, 0, &st, nullptr) != KC_OK) cli::die("decompose");
    *kmax = st.kmax;
    return (int)st.ms;  // integer milliseconds, as the reference returns
}

static void rep_simulation(kc_graph *g, int method, uint32_t *kmax) {
    const int rep = 10;
    float sum = 0;
    unsigned max_time = 0, min_time = UINT32_MAX;
    for (int i = 0; i < rep; i++) {
        const unsigned t = (unsigned)method_run(g, method, kmax);
        std::printf("%ums ", t);
        if (max_time < t) max_time = t;
        if (min_time > t) min_time = t;
        sum += t;
    }
    sum = sum - max_time - min_time;
    std::printf(" ave: %g\n", sum * 1.0 / (rep - 2));
}

int main(int argc, char **argv) {
    if (argc < 2) {
        std::printf("./kcore file deviceID Repeattime\n");
        return -1;
    }
    std::printf("Graph loading Started... \n");
    kc_graph *g = nullptr;
    if (kc_graph_from_mtx(argv[1], KC_LOAD_CSR_DEDUP, 0, &g) != KC_OK) cli::die("load");
    uint32_t n = 0;
    uint64_t nnz = 0;
    uint32_t maxdeg = 0;
    kc_graph_info(g, &n, &nnz, &maxdeg, nullptr);
    std::printf("V: %u\n", n);
    std::printf("E: %llu\n", (unsigned long long)(nnz / 2));
    std::vector<uint32_t> deg(n ? n : 1);
    kc_graph_degrees(g, deg.data());
    double mean = 0;
    for (uint32_t v = 0; v < n; v++) mean += deg[v];
    mean /= n ? n : 1;
    double sq = 0;
    for (uint32_t v = 0; v < n; v++) sq += (deg[v] - mean) * (deg[v] - mean);
    std::printf("\nSTD: \n%g\n", std::sqrt(sq / (n ? n : 1)));
    std::printf(" Maxdegree = %u\n", maxdeg);
    uint32_t kmax = 0;
    std::printf("ICDE23_peel: ");
    rep_simulation(g, KC_PEEL_DYN, &kmax);
    std::printf("Kmax: %u\n", kmax);
    std::printf("Our_Paper_peel: ");
    rep_simulation(g, KC_PEELONE_DYN, &kmax);
    std::printf("Kmax: %u\n", kmax);
    kc_graph_free(g);
    return 0;
}
