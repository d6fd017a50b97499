// The library's minimum-degree ordering, reachable from a test (test
// infrastructure).  The ordering routine is file-local to vgb_host.cpp, so this
// translation unit includes that file and exports one C entry point.
#include "vgb_host.cpp"

// adjacency in CSR form (symmetric, no self loops, sorted rows); writes the
// elimination order (n entries).  Returns 0, or 1 on an exception.
extern "C" int md_order(int n, const int* ptr, const int* idx, int* order) {
    try {
        std::vector<std::vector<int>> adj(n);
        for (int v = 0; v < n; ++v) adj[v].assign(idx + ptr[v], idx + ptr[v + 1]);
        std::vector<int> o = vgb::min_degree_order(n, std::move(adj));
        if ((int)o.size() != n) return 1;
        std::copy(o.begin(), o.end(), order);
        return 0;
    } catch (...) {
        return 1;
    }
}
