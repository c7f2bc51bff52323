// ThreadSanitizer driver for the CPU oracle's threaded paths (test infrastructure only): the
// parallel radix sort, the parallel tree build, the tree walk, counts, FP32 walk and potential,
// the direct sums, the KDK, block and split steps and the direct-sum adjoint, all with 4 worker
// threads on seeded random inputs. Built and run by tests/test_oracle_threads.py with
// -fsanitize=thread; any data race makes ThreadSanitizer report and fail the run.
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

#include "bh_oracle.h"

int main() {
    const int W = 4;
    std::mt19937_64 rng(7);
    std::normal_distribution<double> g(0.0, 1.0);
    std::uniform_int_distribution<uint64_t> u(0, (uint64_t(1) << 63) - 1);

    const int64_t nk = 40000;  // above the oracle's serial threshold
    std::vector<uint64_t> keys(nk);
    std::vector<int32_t> idx(nk);
    for (int64_t i = 0; i < nk; ++i) keys[i] = u(rng), idx[i] = int32_t(i);
    orc_radix_sort_parallel(keys.data(), idx.data(), nk, W);

    const int64_t n = 34000;  // above the threshold of the parallel tree build too
    std::vector<double> px(n), py(n), pz(n), vx(n), vy(n), vz(n), ax(n), ay(n), az(n), m(n, 1.0 / double(n));
    std::vector<uint8_t> kind(n, 0), alive(n, 1);
    for (int64_t i = 0; i < n; ++i) {
        px[i] = g(rng), py[i] = g(rng), pz[i] = g(rng);
        vx[i] = 0.1 * g(rng), vy[i] = 0.1 * g(rng), vz[i] = 0.1 * g(rng);
    }
    orc_tree *t = orc_tree_new();
    orc_tree_build(t, n, px.data(), py.data(), pz.data(), m.data(), kind.data(), alive.data(), 0.5, 8, 0, W);
    orc_tree_accelerations(t, n, 0.01, 0, W, ax.data(), ay.data(), az.data());
    int64_t c[3];
    orc_tree_counts(t, 0.01, 0, W, nullptr, 0, &c[0], &c[1], &c[2]);
    orc_tree_group_counts(t, 64, W, &c[0], &c[1], &c[2]);
    std::vector<float> a32(3 * size_t(n));
    orc_tree_walk_fp32(t, 0.01, W, a32.data());
    double u0 = orc_tree_potential(t, n, px.data(), py.data(), pz.data(), m.data(), kind.data(), alive.data(), 0.01,
                                   0.0, 0, 0, W);
    orc_tree_free(t);
    const int64_t nd = 3000;
    orc_direct(nd, px.data(), py.data(), pz.data(), m.data(), kind.data(), 0.01, 0, W, ax.data(), ay.data(), az.data());
    double ue = orc_potential_exact(nd, px.data(), py.data(), pz.data(), m.data(), kind.data(), 0.01, 0.0, 0, W);
    orc_kdk(n, px.data(), py.data(), pz.data(), vx.data(), vy.data(), vz.data(), ax.data(), ay.data(), az.data(),
            m.data(), kind.data(), alive.data(), 1e-3, 0.01, 0.5, 8, 0, 0, 0, 2, W, 0.0);
    int64_t sub = 0, ev = 0;
    orc_block_kdk(n, px.data(), py.data(), pz.data(), vx.data(), vy.data(), vz.data(), ax.data(), ay.data(), az.data(),
                  m.data(), kind.data(), alive.data(), 4e-3, 0.025, 3, 0.01, 0.5, 8, 0, 0, 1, 1, W, &sub, &ev, 0.0);
    kind[0] = kind[1] = 1;  // two black holes: the split step
    m[0] = m[1] = 0.05;
    orc_split_kdk(n, px.data(), py.data(), pz.data(), vx.data(), vy.data(), vz.data(), ax.data(), ay.data(), az.data(),
                  m.data(), kind.data(), alive.data(), 1e-3, 0.01, 0.5, 8, 0, 0, 0, 2, W, &sub, nullptr, 10.0);
    const int64_t na = 600;
    std::vector<double> gx(na, 1e-3), gv(na, 0.0), d[7];
    for (auto &v : d) v.assign(na, 0.0);
    orc_adjoint_direct(na, px.data(), py.data(), pz.data(), vx.data(), vy.data(), vz.data(), m.data(), 0.01, 1e-3, 6,
                       3, gx.data(), gx.data(), gx.data(), gv.data(), gv.data(), gv.data(), d[0].data(), d[1].data(),
                       d[2].data(), d[3].data(), d[4].data(), d[5].data(), d[6].data(), W);
    std::printf("ok %lld %lld %g %g %lld\n", (long long)c[0], (long long)idx[0], u0, ue, (long long)ev);
    return 0;
}
