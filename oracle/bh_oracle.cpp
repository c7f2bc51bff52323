// bh_oracle.cpp — TEST INFRASTRUCTURE ONLY: the CPU restatement of gravitas'
// Barnes-Hut path used as the parity oracle and as the timed CPU baseline.
// Every function cites the reference file:line it follows. Build with
// -ffp-contract=off (see bh_oracle.h).
#include "bh_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

constexpr int kMortonBits = 21;       // morton.go:4
constexpr int64_t kParallelMin = 1 << 15;  // parallel.go:9
constexpr int kChunksPerWorker = 8;   // sim/parallel.go:10
constexpr int kGrain = 128;           // bh.go:25

int resolve_workers(int workers) {
    if (workers > 0) return workers;
    unsigned h = std::thread::hardware_concurrency();
    return h ? static_cast<int>(h) : 1;
}

// sim/parallel.go:15-40: dynamic chunks of at least grain items.
template <class F>
void parallel_for(int64_t n, int64_t grain, int workers, F fn) {
    workers = resolve_workers(workers);
    if (n <= grain || workers == 1) {
        fn(int64_t(0), n);
        return;
    }
    int64_t chunk = std::max<int64_t>(grain, n / (int64_t(workers) * kChunksPerWorker));
    int64_t chunks = (n + chunk - 1) / chunk;
    std::atomic<int64_t> next{0};
    int nt = static_cast<int>(std::min<int64_t>(workers, chunks));
    std::vector<std::thread> th;
    th.reserve(nt);
    for (int w = 0; w < nt; ++w) {
        th.emplace_back([&] {
            for (;;) {
                int64_t c = next.fetch_add(1);
                if (c >= chunks) return;
                int64_t lo = c * chunk;
                fn(lo, std::min(lo + chunk, n));
            }
        });
    }
    for (auto &t : th) t.join();
}

// parallel.go:14-29: one fixed chunk per worker (serial below parallelMin).
template <class F>
int static_chunks(int64_t n, int workers, F fn) {
    workers = resolve_workers(workers);
    if (n < kParallelMin) workers = 1;
    int64_t chunk = (n + workers - 1) / workers;
    if (workers == 1) {
        fn(0, int64_t(0), n);
        return 1;
    }
    std::vector<std::thread> th;
    for (int w = 0; w < workers; ++w) {
        int64_t lo = std::min<int64_t>(w * chunk, n), hi = std::min<int64_t>((w + 1) * chunk, n);
        th.emplace_back([=, &fn] { fn(w, lo, hi); });
    }
    for (auto &t : th) t.join();
    return workers;
}

// morton.go:7-15.
uint64_t spread(uint64_t v) {
    v &= (uint64_t(1) << kMortonBits) - 1;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}

uint64_t morton_key(uint64_t x, uint64_t y, uint64_t z) {  // morton.go:19-21
    return spread(x) << 2 | spread(y) << 1 | spread(z);
}

// morton.go:25-49.
void radix_sort(uint64_t *keys, int32_t *idx, uint64_t *tmpK, int32_t *tmpI, int64_t n) {
    if (n == 0) return;
    int64_t count[256];
    for (unsigned shift = 0; shift < 64; shift += 8) {
        std::fill(count, count + 256, 0);
        for (int64_t i = 0; i < n; ++i) count[(keys[i] >> shift) & 0xff]++;
        if (count[(keys[0] >> shift) & 0xff] == n) continue;  // all keys share this digit
        int64_t sum = 0;
        for (int d = 0; d < 256; ++d) {
            int64_t c = count[d];
            count[d] = sum;
            sum += c;
        }
        for (int64_t i = 0; i < n; ++i) {
            uint64_t d = (keys[i] >> shift) & 0xff;
            tmpK[count[d]] = keys[i];
            tmpI[count[d]] = idx[i];
            count[d]++;
        }
        std::memcpy(keys, tmpK, n * sizeof(uint64_t));
        std::memcpy(idx, tmpI, n * sizeof(int32_t));
    }
}

// parallel.go:33-88.
void radix_sort_parallel(uint64_t *keys, int32_t *idx, uint64_t *tmpK, int32_t *tmpI, int64_t n,
                         int workers) {
    workers = resolve_workers(workers);
    if (n < kParallelMin || workers == 1) {
        radix_sort(keys, idx, tmpK, tmpI, n);
        return;
    }
    std::vector<std::array<int64_t, 256>> h(workers);
    uint64_t *src = keys, *dst = tmpK;
    int32_t *srcI = idx, *dstI = tmpI;
    for (unsigned shift = 0; shift < 64; shift += 8) {
        static_chunks(n, workers, [&](int w, int64_t lo, int64_t hi) {
            h[w].fill(0);
            for (int64_t i = lo; i < hi; ++i) h[w][(src[i] >> shift) & 0xff]++;
        });
        int64_t total[256] = {};
        for (int w = 0; w < workers; ++w)
            for (int d = 0; d < 256; ++d) total[d] += h[w][d];
        if (total[(src[0] >> shift) & 0xff] == n) continue;
        int64_t sum = 0;  // digit-major, then worker order: the scatter stays stable
        for (int d = 0; d < 256; ++d)
            for (int w = 0; w < workers; ++w) {
                int64_t c = h[w][d];
                h[w][d] = sum;
                sum += c;
            }
        static_chunks(n, workers, [&](int w, int64_t lo, int64_t hi) {
            auto &off = h[w];
            for (int64_t i = lo; i < hi; ++i) {
                uint64_t k = src[i];
                uint64_t d = (k >> shift) & 0xff;
                dst[off[d]] = k;
                dstI[off[d]] = srcI[i];
                off[d]++;
            }
        });
        std::swap(src, dst);
        std::swap(srcI, dstI);
    }
    if (src != keys) {
        std::memcpy(keys, src, n * sizeof(uint64_t));
        std::memcpy(idx, srcI, n * sizeof(int32_t));
    }
}

double offset(int oct, int bit) { return (oct >> bit & 1) == 1 ? 1.0 : -1.0; }  // build.go:353-358

struct Quad {  // build.go:326-337
    double qxx = 0, qyy = 0, qzz = 0, qxy = 0, qxz = 0, qyz = 0;
    void add(double m, double dx, double dy, double dz) {
        double r2 = dx * dx + dy * dy + dz * dz;
        qxx += m * (3 * dx * dx - r2);
        qyy += m * (3 * dy * dy - r2);
        qzz += m * (3 * dz * dz - r2);
        qxy += m * 3 * dx * dy;
        qxz += m * 3 * dx * dz;
        qyz += m * 3 * dy * dz;
    }
};

constexpr int32_t kSubtreeNext = -2;  // build.go:123

}  // namespace

struct orc_tree {
    int leaf = 24;
    double theta = 0.9;
    int workers = 0;
    double minX = 0, minY = 0, minZ = 0, side = 0;
    std::vector<int32_t> order, holes;
    std::vector<uint64_t> keys, tmpK;
    std::vector<int32_t> tmpI;
    std::vector<double> sx, sy, sz, sm;
    std::vector<orc_node> nodes;

    // split build.go:160-172 with lowerBound build.go:340-350.
    int32_t lower_bound(int32_t lo, int32_t hi, unsigned shift, uint64_t oct) const {
        while (lo < hi) {
            int32_t mid = int32_t(uint32_t(lo + hi) >> 1);
            if (((keys[mid] >> shift) & 7) < oct) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    }
    int32_t split(int32_t lo, int32_t hi, int level, int32_t bounds[9]) const {
        unsigned shift = unsigned(3 * (kMortonBits - 1 - level));
        bounds[0] = lo;
        bounds[8] = hi;
        for (uint64_t oct = 1; oct < 8; ++oct) bounds[oct] = lower_bound(bounds[oct - 1], hi, shift, oct);
        int32_t children = 0;
        for (int oct = 0; oct < 8; ++oct)
            if (bounds[oct + 1] > bounds[oct]) children++;
        return children;
    }

    // finish build.go:176-217.
    orc_node finish(const orc_node *nd, int32_t lo, int32_t hi, int32_t first, int32_t children,
                    double cx, double cy, double cz, double half, int32_t next) const {
        double x = 0, y = 0, z = 0, m = 0;
        if (first < 0) {
            for (int32_t j = lo; j < hi; ++j) {
                double mj = sm[j];
                x = x + mj * sx[j];
                y = y + mj * sy[j];
                z = z + mj * sz[j];
                m = m + mj;
            }
        } else {
            for (int32_t c = first; c < first + children; ++c) {
                const orc_node &ch = nd[c];
                x = x + ch.m * ch.x;
                y = y + ch.m * ch.y;
                z = z + ch.m * ch.z;
                m = m + ch.m;
            }
        }
        if (m > 0) {
            x = x / m;
            y = y / m;
            z = z / m;
        } else {
            x = cx;
            y = cy;
            z = cz;
        }
        Quad q;
        if (first < 0) {
            for (int32_t j = lo; j < hi; ++j) q.add(sm[j], sx[j] - x, sy[j] - y, sz[j] - z);
        } else {
            for (int32_t c = first; c < first + children; ++c) {
                const orc_node &ch = nd[c];
                q.qxx = q.qxx + ch.qxx;
                q.qyy = q.qyy + ch.qyy;
                q.qzz = q.qzz + ch.qzz;
                q.qxy = q.qxy + ch.qxy;
                q.qxz = q.qxz + ch.qxz;
                q.qyz = q.qyz + ch.qyz;
                q.add(ch.m, ch.x - x, ch.y - y, ch.z - z);
            }
        }
        double delta = std::sqrt((x - cx) * (x - cx) + (y - cy) * (y - cy) + (z - cz) * (z - cz));
        double crit = 2 * half / theta + delta;
        orc_node out;
        out.x = x;
        out.y = y;
        out.z = z;
        out.m = m;
        out.qxx = q.qxx;
        out.qyy = q.qyy;
        out.qzz = q.qzz;
        out.qxy = q.qxy;
        out.qxz = q.qxz;
        out.qyz = q.qyz;
        out.crit2 = crit * crit;
        out.first = first;
        out.next = next;
        out.lo = lo;
        out.hi = hi;
        return out;
    }

    // buildNode build.go:134-157 into an arbitrary node vector.
    void build_node(std::vector<orc_node> &nd, int32_t ni, int32_t lo, int32_t hi, int level,
                    double cx, double cy, double cz, double half, int32_t next) const {
        int32_t first = -1, children = 0;
        if (hi - lo > leaf && level < kMortonBits) {
            int32_t bounds[9];
            children = split(lo, hi, level, bounds);
            first = int32_t(nd.size());
            nd.resize(nd.size() + children);
            int32_t c = first;
            double q = half / 2;
            for (int oct = 0; oct < 8; ++oct) {
                int32_t clo = bounds[oct], chi = bounds[oct + 1];
                if (chi == clo) continue;
                int32_t child_next = next;
                if (c < first + children - 1) child_next = c + 1;
                build_node(nd, c, clo, chi, level + 1, cx + offset(oct, 2) * q, cy + offset(oct, 1) * q,
                           cz + offset(oct, 0) * q, q, child_next);
                c++;
            }
        }
        nd[ni] = finish(nd.data(), lo, hi, first, children, cx, cy, cz, half, next);
    }

    struct Task {
        int32_t ni, lo, hi;
        int level;
        double cx, cy, cz, half;
        int32_t next;
    };
    struct Top {
        int32_t ni, lo, hi, first, children;
        double cx, cy, cz, half;
        int32_t next;
    };

    // splitTop build.go:299-323.
    void split_top(std::vector<Task> &tasks, std::vector<Top> &tops, int32_t ni, int32_t lo, int32_t hi,
                   int level, double cx, double cy, double cz, double half, int32_t next,
                   int32_t task_size) {
        if (hi - lo <= task_size || hi - lo <= leaf || level >= kMortonBits) {
            tasks.push_back(Task{ni, lo, hi, level, cx, cy, cz, half, next});
            return;
        }
        int32_t bounds[9];
        int32_t children = split(lo, hi, level, bounds);
        int32_t first = int32_t(nodes.size());
        nodes.resize(nodes.size() + children);
        tops.push_back(Top{ni, lo, hi, first, children, cx, cy, cz, half, next});
        int32_t c = first;
        double q = half / 2;
        for (int oct = 0; oct < 8; ++oct) {
            int32_t clo = bounds[oct], chi = bounds[oct + 1];
            if (chi == clo) continue;
            int32_t child_next = next;
            if (c < first + children - 1) child_next = c + 1;
            split_top(tasks, tops, c, clo, chi, level + 1, cx + offset(oct, 2) * q, cy + offset(oct, 1) * q,
                      cz + offset(oct, 0) * q, q, child_next, task_size);
            c++;
        }
    }

    // buildParallel build.go:238-296.
    void build_parallel(int32_t n, double cx, double cy, double cz, double half, int w) {
        int32_t task_size = std::max<int32_t>(8 * leaf, n / int32_t(8 * w));
        std::vector<Task> tasks;
        std::vector<Top> tops;
        nodes.assign(1, orc_node{});
        split_top(tasks, tops, 0, 0, n, 0, cx, cy, cz, half, -1, task_size);
        std::vector<std::vector<orc_node>> locals(tasks.size());
        parallel_for(int64_t(tasks.size()), 1, w, [&](int64_t lo, int64_t hi) {
            for (int64_t ti = lo; ti < hi; ++ti) {
                const Task &task = tasks[ti];
                std::vector<orc_node> &loc = locals[ti];
                loc.assign(1, orc_node{});
                build_node(loc, 0, task.lo, task.hi, task.level, task.cx, task.cy, task.cz, task.half,
                           kSubtreeNext);
            }
        });
        std::vector<int32_t> bases;
        int32_t total = int32_t(nodes.size());
        for (size_t ti = 0; ti < tasks.size(); ++ti) {
            bases.push_back(total);
            total += int32_t(locals[ti].size()) - 1;
        }
        nodes.resize(total);
        parallel_for(int64_t(tasks.size()), 1, w, [&](int64_t lo, int64_t hi) {
            for (int64_t ti = lo; ti < hi; ++ti) {
                const Task &task = tasks[ti];
                int32_t base = bases[ti];
                auto remap = [&](int32_t j) -> int32_t {
                    if (j == kSubtreeNext) return task.next;
                    if (j < 0) return j;
                    if (j == 0) return task.ni;
                    return base + j - 1;
                };
                const std::vector<orc_node> &loc = locals[ti];
                for (size_t j = 0; j < loc.size(); ++j) {
                    orc_node nd = loc[j];
                    nd.first = remap(nd.first);
                    nd.next = remap(nd.next);
                    if (j == 0) nodes[task.ni] = nd;
                    else nodes[base + int32_t(j) - 1] = nd;
                }
            }
        });
        for (int i = int(tops.size()) - 1; i >= 0; --i) {
            const Top &tn = tops[i];
            nodes[tn.ni] = finish(nodes.data(), tn.lo, tn.hi, tn.first, tn.children, tn.cx, tn.cy, tn.cz,
                                  tn.half, tn.next);
        }
    }

    // build.go:11-51 with collect build.go:62-113.
    void build(int64_t n, const double *px, const double *py, const double *pz, const double *mass,
               const uint8_t *kind, const uint8_t *alive, int dm_off) {
        int w = resolve_workers(workers);
        holes.clear();
        order.clear();
        const double inf = std::numeric_limits<double>::infinity();
        double mnX = inf, mnY = inf, mnZ = inf, mxX = -inf, mxY = -inf, mxZ = -inf;
        for (int64_t i = 0; i < n; ++i) {
            bool al = alive[i] != 0;
            if (al && kind[i] == ORC_BLACK_HOLE) holes.push_back(int32_t(i));
            if (!(al && kind[i] != ORC_BLACK_HOLE)) continue;
            order.push_back(int32_t(i));
            mnX = std::min(mnX, px[i]);
            mxX = std::max(mxX, px[i]);
            mnY = std::min(mnY, py[i]);
            mxY = std::max(mxY, py[i]);
            mnZ = std::min(mnZ, pz[i]);
            mxZ = std::max(mxZ, pz[i]);
        }
        nodes.clear();
        int64_t ns = int64_t(order.size());
        minX = mnX;
        minY = mnY;
        minZ = mnZ;
        if (ns == 0) {
            side = 0;
            return;
        }
        double s = std::max(mxX - mnX, std::max(mxY - mnY, mxZ - mnZ));
        s = std::max(s * (1 + 1e-9), 1e-12);
        side = s;
        double scale = double(uint64_t(1) << kMortonBits) / s;
        keys.resize(ns);
        tmpK.resize(ns);
        tmpI.resize(ns);
        auto cell = [&](double v, double lo) -> uint64_t {
            return uint64_t(std::min(double((uint64_t(1) << kMortonBits) - 1), std::max(0.0, (v - lo) * scale)));
        };
        static_chunks(ns, w, [&](int, int64_t lo, int64_t hi) {
            for (int64_t k = lo; k < hi; ++k) {
                int32_t i = order[k];
                keys[k] = morton_key(cell(px[i], mnX), cell(py[i], mnY), cell(pz[i], mnZ));
            }
        });
        radix_sort_parallel(keys.data(), order.data(), tmpK.data(), tmpI.data(), ns, w);
        sx.resize(ns);
        sy.resize(ns);
        sz.resize(ns);
        sm.resize(ns);
        static_chunks(ns, w, [&](int, int64_t lo, int64_t hi) {
            for (int64_t k = lo; k < hi; ++k) {
                int32_t i = order[k];
                sx[k] = px[i];
                sy[k] = py[i];
                sz[k] = pz[i];
                // sim.go:93-98 SourceMass: switched-off dark matter pulls nothing.
                sm[k] = (kind[i] == ORC_DARK_MATTER && dm_off) ? 0.0 : mass[i];
            }
        });
        double half = s / 2;
        if (ns >= kParallelMin && w > 1) {
            build_parallel(int32_t(ns), mnX + half, mnY + half, mnZ + half, half, w);
            return;
        }
        nodes.assign(1, orc_node{});
        build_node(nodes, 0, 0, int32_t(ns), 0, mnX + half, mnY + half, mnZ + half, half, -1);
    }

    // walk bh.go:106-155 (FP64), with optional interaction counts.
    template <bool kCount>
    void walk(double x, double y, double z, int32_t self, double eps2, bool quad, double &oax,
              double &oay, double &oaz, int64_t *cnt) const {
        double ax = 0, ay = 0, az = 0;
        if (nodes.empty()) {
            oax = oay = oaz = 0;
            return;
        }
        const orc_node *nd_ = nodes.data();
        for (int32_t i = 0; i >= 0;) {
            const orc_node &nd = nd_[i];
            double dx = nd.x - x, dy = nd.y - y, dz = nd.z - z;
            double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 >= nd.crit2) {
                double inv = 1 / (d2 + eps2);
                double inv3 = inv * std::sqrt(inv);
                double f = nd.m * inv3;
                if (quad) {
                    double qx = nd.qxx * dx + nd.qxy * dy + nd.qxz * dz;
                    double qy = nd.qxy * dx + nd.qyy * dy + nd.qyz * dz;
                    double qz = nd.qxz * dx + nd.qyz * dy + nd.qzz * dz;
                    double inv5 = inv3 * inv;
                    f += 2.5 * (dx * qx + dy * qy + dz * qz) * inv5 * inv;
                    ax -= qx * inv5;
                    ay -= qy * inv5;
                    az -= qz * inv5;
                }
                ax += f * dx;
                ay += f * dy;
                az += f * dz;
                if (kCount) cnt[0]++;
                i = nd.next;
                continue;
            }
            if (kCount) cnt[2]++;
            if (nd.first >= 0) {
                i = nd.first;
                continue;
            }
            for (int32_t j = nd.lo; j < nd.hi; ++j) {
                if (j == self) continue;
                double ddx = sx[j] - x, ddy = sy[j] - y, ddz = sz[j] - z;
                double r2 = ddx * ddx + ddy * ddy + ddz * ddz + eps2;
                double f = sm[j] / (r2 * std::sqrt(r2));
                ax += f * ddx;
                ay += f * ddy;
                az += f * ddz;
                if (kCount) cnt[1]++;
            }
            i = nd.next;
        }
        oax = ax;
        oay = ay;
        oaz = az;
    }

    // walkPotential potential.go:45-81.
    double walk_potential(double x, double y, double z, int32_t self, double eps2, bool quad) const {
        if (nodes.empty()) return 0;
        double psi = 0;
        const orc_node *nd_ = nodes.data();
        for (int32_t i = 0; i >= 0;) {
            const orc_node &nd = nd_[i];
            double dx = nd.x - x, dy = nd.y - y, dz = nd.z - z;
            double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 >= nd.crit2) {
                double inv = 1 / (d2 + eps2);
                psi += nd.m * std::sqrt(inv);
                if (quad) {
                    double dqd = nd.qxx * dx * dx + nd.qyy * dy * dy + nd.qzz * dz * dz +
                                 2 * (nd.qxy * dx * dy + nd.qxz * dx * dz + nd.qyz * dy * dz);
                    psi += 0.5 * dqd * inv * inv * std::sqrt(inv);
                }
                i = nd.next;
                continue;
            }
            if (nd.first >= 0) {
                i = nd.first;
                continue;
            }
            for (int32_t j = nd.lo; j < nd.hi; ++j) {
                if (j == self) continue;
                double ddx = sx[j] - x, ddy = sy[j] - y, ddz = sz[j] - z;
                psi += sm[j] / std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz + eps2);
            }
            i = nd.next;
        }
        return psi;
    }
};

namespace {

double schwarzschild(double m, double c) { return c <= 0 ? 0 : 2 * m / (c * c); }  // relativity.go:49-54

double gamma_of(double ux, double uy, double uz, double c) {  // relativity.go:15-20
    if (c <= 0) return 1;
    return std::sqrt(1 + (ux * ux + uy * uy + uz * uz) / (c * c));
}

double pair_force(double m, double r2, double eps2, double rs) {  // pair.go:26-35
    double re2 = r2 + eps2;
    double re = std::sqrt(re2);
    if (rs == 0) return m / (re2 * re);
    double den = std::max(re - rs, rs / 2);
    return m / (den * den * re);
}

double pair_rs(uint8_t ki, double mi, uint8_t kj, double mj, double c) {  // pair.go:14-23
    bool hi = ki == ORC_BLACK_HOLE, hj = kj == ORC_BLACK_HOLE;
    if (c <= 0 || hi == hj) return 0;
    if (hi) return schwarzschild(mi, c);
    return schwarzschild(mj, c);
}

double pair_potential(double mi, double mj, double r2, double eps2, double rs) {  // pair.go:37-47
    double re = std::sqrt(r2 + eps2);
    if (rs == 0) return -mi * mj / re;
    if (re >= 1.5 * rs) return -mi * mj / (re - rs);
    return mi * mj * (-2 / rs + 4 / (rs * rs) * (re - 1.5 * rs));
}

double source_mass(uint8_t k, double m, int dm_off) {  // sim.go:93-98
    return (k == ORC_DARK_MATTER && dm_off) ? 0.0 : m;
}

}  // namespace

extern "C" {

uint64_t orc_morton_key(uint64_t x, uint64_t y, uint64_t z) { return morton_key(x, y, z); }

void orc_radix_sort(uint64_t *keys, int32_t *idx, int64_t n) {
    std::vector<uint64_t> tk(n);
    std::vector<int32_t> ti(n);
    radix_sort(keys, idx, tk.data(), ti.data(), n);
}

void orc_radix_sort_parallel(uint64_t *keys, int32_t *idx, int64_t n, int workers) {
    std::vector<uint64_t> tk(n);
    std::vector<int32_t> ti(n);
    radix_sort_parallel(keys, idx, tk.data(), ti.data(), n, workers);
}

orc_tree *orc_tree_new(void) { return new orc_tree(); }
void orc_tree_free(orc_tree *t) { delete t; }

int64_t orc_tree_build(orc_tree *t, int64_t n, const double *px, const double *py, const double *pz,
                       const double *mass, const uint8_t *kind, const uint8_t *alive, double theta,
                       int leaf_size, int dark_matter_off, int workers) {
    t->theta = theta == 0 ? 0.9 : theta;  // bh.go:69-74 (DefaultTheta)
    t->leaf = leaf_size > 0 ? leaf_size : 24;
    t->workers = workers;
    t->build(n, px, py, pz, mass, kind, alive, dark_matter_off);
    return int64_t(t->nodes.size());
}

int64_t orc_tree_nstars(const orc_tree *t) { return int64_t(t->order.size()); }
int64_t orc_tree_nnodes(const orc_tree *t) { return int64_t(t->nodes.size()); }
int64_t orc_tree_nholes(const orc_tree *t) { return int64_t(t->holes.size()); }

void orc_tree_box(const orc_tree *t, double *min3, double *side) {
    min3[0] = t->minX;
    min3[1] = t->minY;
    min3[2] = t->minZ;
    *side = t->side;
}

void orc_tree_export(const orc_tree *t, uint64_t *keys, int32_t *order, orc_node *nodes, double *sx,
                     double *sy, double *sz, double *sm, int32_t *holes) {
    size_t ns = t->order.size();
    if (keys) std::memcpy(keys, t->keys.data(), ns * sizeof(uint64_t));
    if (order) std::memcpy(order, t->order.data(), ns * sizeof(int32_t));
    if (nodes) std::memcpy(nodes, t->nodes.data(), t->nodes.size() * sizeof(orc_node));
    if (sx) std::memcpy(sx, t->sx.data(), ns * sizeof(double));
    if (sy) std::memcpy(sy, t->sy.data(), ns * sizeof(double));
    if (sz) std::memcpy(sz, t->sz.data(), ns * sizeof(double));
    if (sm) std::memcpy(sm, t->sm.data(), ns * sizeof(double));
    if (holes) std::memcpy(holes, t->holes.data(), t->holes.size() * sizeof(int32_t));
}

void orc_tree_accelerations(const orc_tree *t, int64_t n, double eps, int monopole_only, int workers,
                            double *ax, double *ay, double *az) {
    (void)n;
    double eps2 = eps * eps;
    bool quad = !monopole_only;
    parallel_for(int64_t(t->order.size()), kGrain, workers, [&](int64_t lo, int64_t hi) {
        for (int64_t k = lo; k < hi; ++k) {
            int32_t i = t->order[k];
            t->walk<false>(t->sx[k], t->sy[k], t->sz[k], int32_t(k), eps2, quad, ax[i], ay[i], az[i], nullptr);
        }
    });
    for (int32_t i : t->holes) ax[i] = ay[i] = az[i] = 0;  // bh.go:99-101
}

void orc_tree_walk_point(const orc_tree *t, double x, double y, double z, int32_t self, double eps2,
                         int monopole_only, double *a3) {
    t->walk<false>(x, y, z, self, eps2, !monopole_only, a3[0], a3[1], a3[2], nullptr);
}

double orc_tree_walk_potential_point(const orc_tree *t, double x, double y, double z, int32_t self,
                                     double eps2, int monopole_only) {
    return t->walk_potential(x, y, z, self, eps2, !monopole_only);
}

void orc_tree_counts(const orc_tree *t, double eps, int monopole_only, int workers,
                     const int32_t *targets, int64_t ntargets, int64_t *n_node, int64_t *n_pp,
                     int64_t *n_open) {
    double eps2 = eps * eps;
    bool quad = !monopole_only;
    int64_t nt = targets ? ntargets : int64_t(t->order.size());
    std::atomic<int64_t> a{0}, b{0}, c{0};
    parallel_for(nt, kGrain, workers, [&](int64_t lo, int64_t hi) {
        int64_t cnt[3] = {0, 0, 0};
        for (int64_t q = lo; q < hi; ++q) {
            int32_t k = targets ? targets[q] : int32_t(q);
            double x, y, z;
            t->walk<true>(t->sx[k], t->sy[k], t->sz[k], k, eps2, quad, x, y, z, cnt);
        }
        a += cnt[0];
        b += cnt[1];
        c += cnt[2];
    });
    *n_node = a;
    *n_pp = b;
    *n_open = c;
}

// Counts of the group walk the GPU's mixed walk executes: each group of `group` consecutive
// sorted stars walks the tree together and opens a node when any of its stars would (d2 < crit2,
// bh.go:116); every star of the group then takes part in each visit. Same definitions as
// orc_tree_counts (accepted nodes, leaf pairs without the self pair, opened nodes including leaf
// visits), summed over the stars, so group = 1 gives the per-star counts.
void orc_tree_group_counts(const orc_tree *t, int group, int workers, int64_t *n_node, int64_t *n_pp,
                           int64_t *n_open) {
    const int64_t ns = int64_t(t->order.size());
    const int64_t g = group < 1 ? 1 : group;
    const int64_t ng = (ns + g - 1) / g;
    std::atomic<int64_t> a{0}, b{0}, c{0};
    if (!t->nodes.empty()) {
        parallel_for(ng, 16, workers, [&](int64_t lo, int64_t hi) {
            int64_t cnt[3] = {0, 0, 0};
            for (int64_t q = lo; q < hi; ++q) {
                const int64_t s0 = q * g, s1 = s0 + g < ns ? s0 + g : ns, gs = s1 - s0;
                for (int32_t i = 0; i >= 0;) {
                    const orc_node &nd = t->nodes[size_t(i)];
                    bool open = false;
                    for (int64_t k = s0; k < s1 && !open; ++k) {
                        double dx = nd.x - t->sx[size_t(k)], dy = nd.y - t->sy[size_t(k)], dz = nd.z - t->sz[size_t(k)];
                        open = dx * dx + dy * dy + dz * dz < nd.crit2;
                    }
                    if (!open) {
                        cnt[0] += gs;
                        i = nd.next;
                        continue;
                    }
                    cnt[2] += gs;
                    if (nd.first >= 0) {
                        i = nd.first;
                        continue;
                    }
                    const int64_t l0 = s0 > nd.lo ? s0 : int64_t(nd.lo), l1 = s1 < nd.hi ? s1 : int64_t(nd.hi);
                    cnt[1] += gs * int64_t(nd.hi - nd.lo) - (l1 > l0 ? l1 - l0 : 0);  // no self pairs
                    i = nd.next;
                }
            }
            a += cnt[0];
            b += cnt[1];
            c += cnt[2];
        });
    }
    *n_node = a;
    *n_pp = b;
    *n_open = c;
}

// gpu_darwin.go:84-117 with the float32 packing of :187-202, on the CPU.
void orc_tree_walk_fp32(const orc_tree *t, double eps, int workers, float *acc3) {
    struct GNode {
        float com[4], q1[4], q2[4];
        int32_t links[4];
    };
    size_t nn = t->nodes.size(), ns = t->order.size();
    std::vector<GNode> g(nn);
    for (size_t i = 0; i < nn; ++i) {
        const orc_node &nd = t->nodes[i];
        g[i] = GNode{{float(nd.x), float(nd.y), float(nd.z), float(nd.m)},
                     {float(nd.qxx), float(nd.qyy), float(nd.qzz), float(nd.qxy)},
                     {float(nd.qxz), float(nd.qyz), float(nd.crit2), 0.f},
                     {nd.first, nd.next, nd.lo, nd.hi}};
    }
    std::vector<float> st(4 * ns);
    for (size_t k = 0; k < ns; ++k) {
        st[4 * k] = float(t->sx[k]);
        st[4 * k + 1] = float(t->sy[k]);
        st[4 * k + 2] = float(t->sz[k]);
        st[4 * k + 3] = float(t->sm[k]);
    }
    float eps2 = float(eps * eps);
    parallel_for(int64_t(ns), 8192, workers, [&](int64_t lo, int64_t hi) {
        for (int64_t k = lo; k < hi; ++k) {
            float px = st[4 * k], py = st[4 * k + 1], pz = st[4 * k + 2];
            float ax = 0, ay = 0, az = 0;
            int i = nn ? 0 : -1;
            while (i >= 0) {
                const GNode &nd = g[i];
                float dx = nd.com[0] - px, dy = nd.com[1] - py, dz = nd.com[2] - pz;
                float d2 = dx * dx + dy * dy + dz * dz;
                if (d2 >= nd.q2[2]) {
                    float inv = 1.0f / (d2 + eps2);
                    float inv3 = inv * std::sqrt(inv);
                    float qx = nd.q1[0] * dx + nd.q1[3] * dy + nd.q2[0] * dz;
                    float qy = nd.q1[3] * dx + nd.q1[1] * dy + nd.q2[1] * dz;
                    float qz = nd.q2[0] * dx + nd.q2[1] * dy + nd.q1[2] * dz;
                    float inv5 = inv3 * inv;
                    float f = nd.com[3] * inv3 + 2.5f * (dx * qx + dy * qy + dz * qz) * inv5 * inv;
                    ax += dx * f - qx * inv5;
                    ay += dy * f - qy * inv5;
                    az += dz * f - qz * inv5;
                    i = nd.links[1];
                    continue;
                }
                if (nd.links[0] >= 0) {
                    i = nd.links[0];
                    continue;
                }
                for (int j = nd.links[2]; j < nd.links[3]; ++j) {
                    if (j == int(k)) continue;
                    float ddx = st[4 * j] - px, ddy = st[4 * j + 1] - py, ddz = st[4 * j + 2] - pz;
                    float ir = 1.0f / std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz + eps2);
                    float f = st[4 * j + 3] * ir * ir * ir;
                    ax += ddx * f;
                    ay += ddy * f;
                    az += ddz * f;
                }
                i = nd.links[1];
            }
            acc3[3 * k] = ax;
            acc3[3 * k + 1] = ay;
            acc3[3 * k + 2] = az;
        }
    });
}

double orc_tree_potential(const orc_tree *t, int64_t n, const double *px, const double *py,
                          const double *pz, const double *mass, const uint8_t *kind,
                          const uint8_t *alive, double eps, double c, int dm_off, int monopole_only,
                          int workers) {
    (void)n;
    (void)alive;
    double eps2 = eps * eps;
    bool quad = !monopole_only;
    const auto &holes = t->holes;
    // holePotential potential.go:84-96.
    auto hole_potential = [&](int32_t i) {
        double x = px[i], y = py[i], z = pz[i], u = 0;
        for (int32_t h : holes) {
            if (h == i) continue;
            double dx = px[h] - x, dy = py[h] - y, dz = pz[h] - z;
            double rs = pair_rs(kind[i], mass[i], ORC_BLACK_HOLE, mass[h], c);
            u += pair_potential(source_mass(kind[i], mass[i], dm_off), mass[h], dx * dx + dy * dy + dz * dz,
                                eps2, rs);
        }
        return u;
    };
    int64_t ns = int64_t(t->order.size());
    // potential.go:21-30; chunk parts are summed in chunk order (the reference sums them in
    // completion order, so only round-off may differ).
    int64_t chunk = 4096;
    int64_t nch = (ns + chunk - 1) / chunk;
    std::vector<double> parts(nch, 0.0);
    parallel_for(nch, 1, workers, [&](int64_t lo, int64_t hi) {
        for (int64_t ci = lo; ci < hi; ++ci) {
            double part = 0;
            for (int64_t k = ci * chunk; k < std::min(ns, (ci + 1) * chunk); ++k) {
                int32_t i = t->order[k];
                part += t->sm[k] * t->walk_potential(t->sx[k], t->sy[k], t->sz[k], int32_t(k), eps2, quad) -
                        hole_potential(i);
            }
            parts[ci] = part;
        }
    });
    double sum = 0;
    for (double p : parts) sum += p;
    for (int32_t i : holes) {  // potential.go:32-40
        double x = px[i], y = py[i], z = pz[i];
        double rs = schwarzschild(mass[i], c);
        for (int64_t k = 0; k < ns; ++k) {
            double dx = t->sx[k] - x, dy = t->sy[k] - y, dz = t->sz[k] - z;
            sum -= pair_potential(mass[i], t->sm[k], dx * dx + dy * dy + dz * dz, eps2, rs);
        }
        sum -= hole_potential(i);
    }
    return -sum / 2;
}

static void direct_one(int64_t n, const double *px, const double *py, const double *pz, const double *m,
                       const uint8_t *kind, double eps2, int dm_off, int64_t i, double &oax, double &oay,
                       double &oaz) {
    // direct.go:27-47.
    double xi = px[i], yi = py[i], zi = pz[i];
    double ax = 0, ay = 0, az = 0;
    if (kind[i] == ORC_BLACK_HOLE) {
        oax = oay = oaz = 0;
        return;
    }
    for (int64_t j = 0; j < n; ++j) {
        if (j == i || kind[j] == ORC_BLACK_HOLE || (dm_off && kind[j] == ORC_DARK_MATTER)) continue;
        double dx = px[j] - xi, dy = py[j] - yi, dz = pz[j] - zi;
        double re2 = dx * dx + dy * dy + dz * dz + eps2;
        double f = m[j] / (re2 * std::sqrt(re2));
        ax += f * dx;
        ay += f * dy;
        az += f * dz;
    }
    oax = ax;
    oay = ay;
    oaz = az;
}

void orc_direct(int64_t n, const double *px, const double *py, const double *pz, const double *mass,
                const uint8_t *kind, double eps, int dm_off, int workers, double *ax, double *ay,
                double *az) {
    double eps2 = eps * eps;
    parallel_for(n, 64, workers, [&](int64_t lo, int64_t hi) {  // direct.go:11,20-21
        for (int64_t i = lo; i < hi; ++i) direct_one(n, px, py, pz, mass, kind, eps2, dm_off, i, ax[i], ay[i], az[i]);
    });
}

void orc_direct_targets(int64_t n, const double *px, const double *py, const double *pz,
                        const double *mass, const uint8_t *kind, double eps, int dm_off,
                        const int64_t *targets, int64_t ntargets, int workers, double *ax, double *ay,
                        double *az) {
    double eps2 = eps * eps;
    parallel_for(ntargets, 4, workers, [&](int64_t lo, int64_t hi) {
        for (int64_t q = lo; q < hi; ++q)
            direct_one(n, px, py, pz, mass, kind, eps2, dm_off, targets[q], ax[q], ay[q], az[q]);
    });
}

void orc_kdk(int64_t n, double *px, double *py, double *pz, double *vx, double *vy, double *vz,
             double *ax, double *ay, double *az, const double *mass, const uint8_t *kind,
             const uint8_t *alive, double dt, double eps, double theta, int leaf_size, int monopole_only,
             int dm_off, int acc_valid, int64_t nsteps, int workers, double c) {
    orc_tree t;
    t.theta = theta == 0 ? 0.9 : theta;
    t.leaf = leaf_size > 0 ? leaf_size : 24;
    t.workers = workers;
    auto forces = [&] {
        t.build(n, px, py, pz, mass, kind, alive, dm_off);
        orc_tree_accelerations(&t, n, eps, monopole_only, workers, ax, ay, az);
    };
    if (!acc_valid) forces();  // gas.go:14-17 (initForces)
    double h = 0.5 * dt;
    for (int64_t s = 0; s < nsteps; ++s) {
        for (int64_t i = 0; i < n; ++i) {  // kick sim.go:302-311
            vx[i] += h * ax[i];
            vy[i] += h * ay[i];
            vz[i] += h * az[i];
        }
        if (c <= 0) {
            for (int64_t i = 0; i < n; ++i) {  // drift sim.go:327-334
                px[i] += dt * vx[i];
                py[i] += dt * vy[i];
                pz[i] += dt * vz[i];
            }
        } else {
            const double inv_c2 = 1 / (c * c);
            for (int64_t i = 0; i < n; ++i) {  // drift sim.go:335-343: the coordinate velocity u / gamma
                double ux = vx[i], uy = vy[i], uz = vz[i];
                double f = dt / std::sqrt(1 + (ux * ux + uy * uy + uz * uz) * inv_c2);
                px[i] += f * ux;
                py[i] += f * uy;
                pz[i] += f * uz;
            }
        }
        forces();  // advanceGas without gas: Solver.Accelerations (blockstep.go:129-135)
        for (int64_t i = 0; i < n; ++i) {
            vx[i] += h * ax[i];
            vy[i] += h * ay[i];
            vz[i] += h * az[i];
        }
    }
}

namespace {

constexpr double kNearSteps = 20.0;      // split.go:18-19
constexpr double kSubstepsPerTau = 20.0;  // split.go:20-21
constexpr int kMaxSubsteps = 256;         // split.go:22-23
constexpr int64_t kHoleChunk = 256;       // bodies per partial sum of a hole's far-star pull


}  // namespace

void orc_split_kdk(int64_t n, double *px, double *py, double *pz, double *vx, double *vy, double *vz, double *ax,
                   double *ay, double *az, const double *mass, const uint8_t *kind, const uint8_t *alive, double dt,
                   double eps, double theta, int leaf_size, int monopole_only, int dm_off, int acc_valid,
                   int64_t nsteps, int workers, int64_t *substeps, uint8_t *near_out, double c) {
    orc_tree t;
    t.theta = theta == 0 ? 0.9 : theta;
    t.leaf = leaf_size > 0 ? leaf_size : 24;
    t.workers = workers;
    auto forces = [&] {
        t.build(n, px, py, pz, mass, kind, alive, dm_off);
        orc_tree_accelerations(&t, n, eps, monopole_only, workers, ax, ay, az);
    };
    if (!acc_valid) forces();
    const double eps2 = eps * eps, h = 0.5 * dt;
    auto is_hole = [&](int64_t i) { return kind && kind[i] == ORC_BLACK_HOLE; };
    auto src_mass = [&](int64_t i) { return dm_off && kind && kind[i] == ORC_DARK_MATTER ? 0.0 : mass[i]; };
    std::vector<int64_t> holes, near;
    std::vector<uint8_t> is_near(size_t(n), 0);
    std::vector<double> far(3 * size_t(n)), fast(3 * size_t(n));
    auto kind_of = [&](int64_t i) -> uint8_t { return kind ? kind[i] : uint8_t(ORC_STAR); };
    // split.go:27-36
    auto timescale = [&](int64_t i, int64_t hh) {
        double dx = px[i] - px[hh], dy = py[i] - py[hh], dz = pz[i] - pz[hh];
        double r2 = dx * dx + dy * dy + dz * dz;
        double rs = pair_rs(kind_of(i), mass[i], ORC_BLACK_HOLE, mass[hh], c);
        double a = pair_force(mass[hh], r2, eps2, rs) * std::sqrt(r2);
        if (a == 0) return std::numeric_limits<double>::infinity();
        return std::sqrt(std::sqrt(r2 + eps2) / a);
    };
    // holePull, split.go:119-137
    auto hole_pull = [&](int64_t i, double &fx, double &fy, double &fz) {
        fx = fy = fz = 0;
        for (int64_t hh : holes) {
            if (hh == i) continue;
            double dx = px[hh] - px[i], dy = py[hh] - py[i], dz = pz[hh] - pz[i];
            double rs = pair_rs(kind_of(i), mass[i], ORC_BLACK_HOLE, mass[hh], c);
            double f = pair_force(mass[hh], dx * dx + dy * dy + dz * dz, eps2, rs);
            fx += f * dx;
            fy += f * dy;
            fz += f * dz;
        }
    };
    // outerHoleForces, split.go:83-117
    auto outer = [&] {
        std::fill(far.begin(), far.end(), 0.0);
        parallel_for(n, kGrain, workers, [&](int64_t lo, int64_t hi) {
            for (int64_t i = lo; i < hi; ++i)
                if (!is_hole(i) && !is_near[size_t(i)]) hole_pull(i, far[size_t(i)], far[size_t(n + i)], far[size_t(2 * n + i)]);
        });
        for (int64_t hh : holes) {
            double x = px[hh], y = py[hh], z = pz[hh];
            double rs = schwarzschild(mass[hh], c);
            for (int64_t c0 = 0; c0 < n; c0 += kHoleChunk) {
                double sx = 0, sy = 0, sz = 0;
                for (int64_t i = c0; i < std::min(n, c0 + kHoleChunk); ++i) {
                    if (is_hole(i) || is_near[size_t(i)]) continue;
                    double dx = px[i] - x, dy = py[i] - y, dz = pz[i] - z;
                    double f = pair_force(src_mass(i), dx * dx + dy * dy + dz * dz, eps2, rs);
                    sx += f * dx;
                    sy += f * dy;
                    sz += f * dz;
                }
                far[size_t(hh)] += sx;
                far[size_t(n + hh)] += sy;
                far[size_t(2 * n + hh)] += sz;
            }
        }
    };
    // fastForces, split.go:139-159
    auto fast_forces = [&] {
        for (int64_t i : near) hole_pull(i, fast[size_t(i)], fast[size_t(n + i)], fast[size_t(2 * n + i)]);
        for (int64_t hh : holes) {
            double x = px[hh], y = py[hh], z = pz[hh];
            double rs = schwarzschild(mass[hh], c);
            double sx, sy, sz;
            hole_pull(hh, sx, sy, sz);
            for (int64_t i : near) {
                double dx = px[i] - x, dy = py[i] - y, dz = pz[i] - z;
                double f = pair_force(src_mass(i), dx * dx + dy * dy + dz * dz, eps2, rs);
                sx += f * dx;
                sy += f * dy;
                sz += f * dz;
            }
            fast[size_t(hh)] = sx;
            fast[size_t(n + hh)] = sy;
            fast[size_t(2 * n + hh)] = sz;
        }
    };
    auto kick_outer = [&](double k) {  // split.go:206-213
        for (int64_t i = 0; i < n; ++i) {
            vx[i] += k * (ax[i] + far[size_t(i)]);
            vy[i] += k * (ay[i] + far[size_t(n + i)]);
            vz[i] += k * (az[i] + far[size_t(2 * n + i)]);
        }
    };
    auto kick_fast = [&](double k) {  // split.go:215-224
        for (const auto *idx : {&near, &holes})
            for (int64_t i : *idx) {
                vx[i] += k * fast[size_t(i)];
                vy[i] += k * fast[size_t(n + i)];
                vz[i] += k * fast[size_t(2 * n + i)];
            }
    };
    auto drift_idx = [&](const std::vector<int64_t> &idx, double d) {  // split.go:226-234
        for (int64_t i : idx) {
            double f = d / gamma_of(vx[i], vy[i], vz[i], c);
            px[i] += f * vx[i];
            py[i] += f * vy[i];
            pz[i] += f * vz[i];
        }
    };
    int64_t last = 1;
    for (int64_t step = 0; step < nsteps; ++step) {
        holes.clear();
        for (int64_t i = 0; i < n; ++i)  // collectHoles, sim.go:294-302
            if ((!alive || alive[i]) && is_hole(i)) holes.push_back(i);
        if (holes.empty()) {  // sim.go:266-280
            std::fill(is_near.begin(), is_near.end(), 0);
            for (int64_t i = 0; i < n; ++i) {
                vx[i] += h * ax[i];
                vy[i] += h * ay[i];
                vz[i] += h * az[i];
            }
            const double inv_c2 = c > 0 ? 1 / (c * c) : 0;
            for (int64_t i = 0; i < n; ++i) {  // drift sim.go:315-343
                double f = dt;
                if (c > 0) f = dt / std::sqrt(1 + (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]) * inv_c2);
                px[i] += f * vx[i];
                py[i] += f * vy[i];
                pz[i] += f * vz[i];
            }
            forces();
            for (int64_t i = 0; i < n; ++i) {
                vx[i] += h * ax[i];
                vy[i] += h * ay[i];
                vz[i] += h * az[i];
            }
            last = 1;
            continue;
        }
        // classify, split.go:39-85
        const double limit = kNearSteps * dt;
        double tau_min = std::numeric_limits<double>::infinity();
        for (int64_t i = 0; i < n; ++i) {
            bool nr = false;
            if (!is_hole(i))
                for (int64_t hh : holes) {
                    double tau = timescale(i, hh);
                    if (tau < limit) nr = true, tau_min = std::min(tau_min, tau);
                }
            is_near[size_t(i)] = nr;
        }
        for (size_t a = 0; a < holes.size(); ++a)
            for (size_t b = a + 1; b < holes.size(); ++b) {
                double tau = timescale(holes[a], holes[b]);
                if (tau < limit) tau_min = std::min(tau_min, tau);
            }
        near.clear();
        for (int64_t i = 0; i < n; ++i)
            if (is_near[size_t(i)]) near.push_back(i);
        int64_t k = 1;
        if (!std::isinf(tau_min))
            while (double(k) * tau_min < kSubstepsPerTau * dt && k < kMaxSubsteps) k *= 2;
        last = k;
        // stepSplit, split.go:162-200 (c = 0, no gas, no spin)
        outer();
        kick_outer(h);
        const double hs = dt / double(k);
        fast_forces();
        for (int64_t q = 0; q < k; ++q) {
            kick_fast(0.5 * hs);
            drift_idx(near, hs);
            drift_idx(holes, hs);
            fast_forces();
            kick_fast(0.5 * hs);
        }
        for (int64_t i = 0; i < n; ++i) {  // driftFar
            if (is_hole(i) || is_near[size_t(i)]) continue;
            double f = dt / gamma_of(vx[i], vy[i], vz[i], c);
            px[i] += f * vx[i];
            py[i] += f * vy[i];
            pz[i] += f * vz[i];
        }
        forces();  // advanceGas without gas
        outer();
        kick_outer(h);
    }
    if (substeps) *substeps = last;
    if (near_out)
        for (int64_t i = 0; i < n; ++i) near_out[i] = is_near[size_t(i)];
}

void orc_block_kdk(int64_t n, double *px, double *py, double *pz, double *vx, double *vy, double *vz, double *ax,
                   double *ay, double *az, const double *mass, const uint8_t *kind, const uint8_t *alive, double T,
                   double eta, int levels, double eps, double theta, int leaf_size, int monopole_only, int dm_off,
                   int acc_valid, int64_t nsteps, int workers, int64_t *substeps, int64_t *evals, double c) {
    orc_tree t;
    t.theta = theta == 0 ? 0.9 : theta;
    t.leaf = leaf_size > 0 ? leaf_size : 24;
    t.workers = workers;
    double eps2 = eps * eps;
    bool quad = !monopole_only;
    if (!acc_valid) {
        t.build(n, px, py, pz, mass, kind, alive, dm_off);
        orc_tree_accelerations(&t, n, eps, monopole_only, workers, ax, ay, az);
    }
    const int32_t ticks = 1 << (levels - 1);
    auto rung_for = [&](double dt) {  // blockstep.go:38-45
        int r = 0;
        double x = T;
        while (x > dt && r < levels - 1) {
            x *= 0.5;
            ++r;
        }
        return r;
    };
    auto body_dt = [&](int64_t i) {
        double a = std::sqrt(ax[i] * ax[i] + ay[i] * ay[i] + az[i] * az[i]);
        return a > 0 ? eta * std::sqrt(eps / a) : std::numeric_limits<double>::infinity();
    };
    std::vector<int> rung(n);
    std::vector<int32_t> end(n);
    int64_t ns = 0, ne = 0;
    for (int64_t s = 0; s < nsteps; ++s) {
        int32_t next = std::numeric_limits<int32_t>::max();
        for (int64_t i = 0; i < n; ++i) {  // tick 0: every body opens a step
            int r = rung_for(body_dt(i));
            rung[i] = r;
            end[i] = ticks >> r;
            double h = 0.5 * (T / double(1 << r));
            vx[i] += h * ax[i];
            vy[i] += h * ay[i];
            vz[i] += h * az[i];
            next = std::min(next, end[i]);
        }
        int32_t tk = 0;
        while (tk < ticks) {
            int32_t tn = next;
            double d = double(tn - tk) * (T / double(ticks));
            for (int64_t i = 0; i < n; ++i) {
                double f = d / gamma_of(vx[i], vy[i], vz[i], c);  // driftOne, sim.go:345-350
                px[i] += f * vx[i];
                py[i] += f * vy[i];
                pz[i] += f * vz[i];
            }
            tk = tn;
            t.build(n, px, py, pz, mass, kind, alive, dm_off);
            for (int32_t h : t.holes) ax[h] = ay[h] = az[h] = 0;
            std::vector<int64_t> act;
            for (int64_t k = 0; k < int64_t(t.order.size()); ++k)
                if (end[t.order[k]] == tk) act.push_back(k);
            parallel_for(int64_t(act.size()), kGrain, workers, [&](int64_t lo, int64_t hi) {
                for (int64_t q = lo; q < hi; ++q) {
                    int64_t k = act[q];
                    int32_t i = t.order[k];
                    t.walk<false>(t.sx[k], t.sy[k], t.sz[k], int32_t(k), eps2, quad, ax[i], ay[i], az[i], nullptr);
                }
            });
            ++ns;
            ne += int64_t(act.size());
            next = std::numeric_limits<int32_t>::max();
            for (int64_t i = 0; i < n; ++i) {
                if (end[i] == tk) {
                    double h = 0.5 * (T / double(1 << rung[i]));
                    vx[i] += h * ax[i];
                    vy[i] += h * ay[i];
                    vz[i] += h * az[i];
                    if (tk < ticks) {
                        int r = rung_for(body_dt(i));
                        while (tk % (ticks >> r) != 0) ++r;
                        rung[i] = r;
                        end[i] = tk + (ticks >> r);
                        double h2 = 0.5 * (T / double(1 << r));
                        vx[i] += h2 * ax[i];
                        vy[i] += h2 * ay[i];
                        vz[i] += h2 * az[i];
                    }
                }
                next = std::min(next, end[i]);
            }
        }
    }
    if (substeps) *substeps = ns;
    if (evals) *evals = ne;
}

namespace {

// Direct-sum accelerations of all bodies (all stars), j in index order (direct.go:27-47).
void direct_all(int64_t n, const double *px, const double *py, const double *pz, const double *m, double eps2,
                int workers, double *ax, double *ay, double *az) {
    parallel_for(n, 64, workers, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            double xi = px[i], yi = py[i], zi = pz[i], fx = 0, fy = 0, fz = 0;
            for (int64_t j = 0; j < n; ++j) {
                if (j == i) continue;
                double dx = px[j] - xi, dy = py[j] - yi, dz = pz[j] - zi;
                double re2 = dx * dx + dy * dy + dz * dz + eps2;
                double f = m[j] / (re2 * std::sqrt(re2));
                fx += f * dx;
                fy += f * dy;
                fz += f * dz;
            }
            ax[i] = fx;
            ay[i] = fy;
            az[i] = fz;
        }
    });
}

// Vector-Jacobian product of the direct-sum accelerations a(x; m) with weights w:
//   g_x[i] = sum_j (da_j/dx_i)^T w_j = sum_{j != i} K(d) (m_i w_j - m_j w_i),
//   g_m[i] = sum_j (da_j/dm_i) . w_j = -sum_{j != i} (w_j . d) / s^3,
// with d = x_j - x_i, s^2 = |d|^2 + eps^2, K(d) = I / s^3 - 3 d d^T / s^5. Adds c * g to (gx, gm).
void vjp_all(int64_t n, const double *px, const double *py, const double *pz, const double *m, const double *wx,
             const double *wy, const double *wz, double eps2, double c, int workers, double *gx, double *gy,
             double *gz, double *gm) {
    parallel_for(n, 64, workers, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            double xi = px[i], yi = py[i], zi = pz[i], mi = m[i];
            double wix = wx[i], wiy = wy[i], wiz = wz[i];
            double sx = 0, sy = 0, sz = 0, sm = 0;
            for (int64_t j = 0; j < n; ++j) {
                if (j == i) continue;
                double dx = px[j] - xi, dy = py[j] - yi, dz = pz[j] - zi;
                double s2 = dx * dx + dy * dy + dz * dz + eps2;
                double inv3 = 1 / (s2 * std::sqrt(s2));
                double inv5 = inv3 / s2;
                double ux = mi * wx[j] - m[j] * wix, uy = mi * wy[j] - m[j] * wiy, uz = mi * wz[j] - m[j] * wiz;
                double du = dx * ux + dy * uy + dz * uz;
                sx += ux * inv3 - 3 * dx * du * inv5;
                sy += uy * inv3 - 3 * dy * du * inv5;
                sz += uz * inv3 - 3 * dz * du * inv5;
                sm -= (wx[j] * dx + wy[j] * dy + wz[j] * dz) * inv3;
            }
            gx[i] += c * sx;
            gy[i] += c * sy;
            gz[i] += c * sz;
            gm[i] += c * sm;
        }
    });
}

}  // namespace

void orc_kdk_direct(int64_t n, double *px, double *py, double *pz, double *vx, double *vy, double *vz,
                    const double *mass, double eps, double dt, int64_t nsteps, int workers) {
    std::vector<double> ax(n), ay(n), az(n);
    double eps2 = eps * eps, h = 0.5 * dt;
    direct_all(n, px, py, pz, mass, eps2, workers, ax.data(), ay.data(), az.data());
    for (int64_t s = 0; s < nsteps; ++s) {
        for (int64_t i = 0; i < n; ++i) {
            vx[i] += h * ax[i];
            vy[i] += h * ay[i];
            vz[i] += h * az[i];
            px[i] += dt * vx[i];
            py[i] += dt * vy[i];
            pz[i] += dt * vz[i];
        }
        direct_all(n, px, py, pz, mass, eps2, workers, ax.data(), ay.data(), az.data());
        for (int64_t i = 0; i < n; ++i) {
            vx[i] += h * ax[i];
            vy[i] += h * ay[i];
            vz[i] += h * az[i];
        }
    }
}

void orc_adjoint_direct(int64_t n, const double *px, const double *py, const double *pz, const double *vx,
                        const double *vy, const double *vz, const double *mass, double eps, double dt, int64_t nsteps,
                        int64_t every, const double *gx, const double *gy, const double *gz, const double *gvx,
                        const double *gvy, const double *gvz, double *dx, double *dy, double *dz, double *dvx,
                        double *dvy, double *dvz, double *dm, int workers) {
    const double eps2 = eps * eps, h = 0.5 * dt;
    if (every < 1) every = 1;
    // forward: checkpoints of (x, v) at steps 0, every, 2 every, ...
    std::vector<std::vector<double>> ck;
    std::vector<double> x(px, px + n), y(py, py + n), z(pz, pz + n), u(vx, vx + n), v(vy, vy + n), w(vz, vz + n);
    for (int64_t s0 = 0; s0 < nsteps; s0 += every) {
        std::vector<double> c(6 * n);
        for (int64_t i = 0; i < n; ++i) {
            c[i] = x[i];
            c[n + i] = y[i];
            c[2 * n + i] = z[i];
            c[3 * n + i] = u[i];
            c[4 * n + i] = v[i];
            c[5 * n + i] = w[i];
        }
        ck.push_back(std::move(c));
        int64_t k = std::min(every, nsteps - s0);
        orc_kdk_direct(n, x.data(), y.data(), z.data(), u.data(), v.data(), w.data(), mass, eps, dt, k, workers);
    }
    // backward
    std::vector<double> lx(gx, gx + n), ly(gy, gy + n), lz(gz, gz + n), lu(gvx, gvx + n), lv(gvy, gvy + n),
        lw(gvz, gvz + n), lm(n, 0.0);
    // closing kick of the last step, at the final positions
    vjp_all(n, x.data(), y.data(), z.data(), mass, lu.data(), lv.data(), lw.data(), eps2, h, workers, lx.data(),
            ly.data(), lz.data(), lm.data());
    for (int64_t c = int64_t(ck.size()) - 1; c >= 0; --c) {
        int64_t s0 = c * every, k = std::min(every, nsteps - s0);
        // replay the segment, keeping the positions at its step starts
        std::vector<std::vector<double>> pos(k);
        std::vector<double> sx(ck[c].begin(), ck[c].begin() + n), sy(ck[c].begin() + n, ck[c].begin() + 2 * n),
            sz(ck[c].begin() + 2 * n, ck[c].begin() + 3 * n), su(ck[c].begin() + 3 * n, ck[c].begin() + 4 * n),
            sv(ck[c].begin() + 4 * n, ck[c].begin() + 5 * n), sw(ck[c].begin() + 5 * n, ck[c].end());
        for (int64_t q = 0; q < k; ++q) {
            pos[q].resize(3 * n);
            std::copy(sx.begin(), sx.end(), pos[q].begin());
            std::copy(sy.begin(), sy.end(), pos[q].begin() + n);
            std::copy(sz.begin(), sz.end(), pos[q].begin() + 2 * n);
            if (q + 1 < k)
                orc_kdk_direct(n, sx.data(), sy.data(), sz.data(), su.data(), sv.data(), sw.data(), mass, eps, dt, 1,
                               workers);
        }
        for (int64_t q = k - 1; q >= 0; --q) {
            int64_t s = s0 + q;
            for (int64_t i = 0; i < n; ++i) {  // drift x_{s+1} = x_s + dt v_half
                lu[i] += dt * lx[i];
                lv[i] += dt * ly[i];
                lw[i] += dt * lz[i];
            }
            // opening kick of step s and closing kick of step s-1 act at x_s with the same weights
            double cf = s > 0 ? dt : h;
            const double *P = pos[q].data();
            vjp_all(n, P, P + n, P + 2 * n, mass, lu.data(), lv.data(), lw.data(), eps2, cf, workers, lx.data(),
                    ly.data(), lz.data(), lm.data());
        }
    }
    std::copy(lx.begin(), lx.end(), dx);
    std::copy(ly.begin(), ly.end(), dy);
    std::copy(lz.begin(), lz.end(), dz);
    std::copy(lu.begin(), lu.end(), dvx);
    std::copy(lv.begin(), lv.end(), dvy);
    std::copy(lw.begin(), lw.end(), dvz);
    std::copy(lm.begin(), lm.end(), dm);
}

double orc_pair_force(double m, double r2, double eps2, double rs) { return pair_force(m, r2, eps2, rs); }
double orc_pair_potential(double mi, double mj, double r2, double eps2, double rs) {
    return pair_potential(mi, mj, r2, eps2, rs);
}
double orc_pair_rs(uint8_t ki, double mi, uint8_t kj, double mj, double c) { return pair_rs(ki, mi, kj, mj, c); }

double orc_potential_exact(int64_t n, const double *px, const double *py, const double *pz,
                           const double *mass, const uint8_t *kind, double eps, double c, int dm_off,
                           int workers) {
    // diag.go:42-64: each row i summed over j > i ascending, the rows added in ascending i (the
    // reference adds its ParallelFor chunks in completion order, so only round-off may differ).
    double eps2 = eps * eps;
    std::vector<double> rows(size_t(std::max<int64_t>(n, 0)), 0.0);
    parallel_for(n, 64, workers, [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) {
            double xi = px[i], yi = py[i], zi = pz[i], part = 0;
            for (int64_t j = i + 1; j < n; ++j) {
                double dx = px[j] - xi, dy = py[j] - yi, dz = pz[j] - zi;
                double rs = pair_rs(kind[i], mass[i], kind[j], mass[j], c);
                part += pair_potential(source_mass(kind[i], mass[i], dm_off), source_mass(kind[j], mass[j], dm_off),
                                       dx * dx + dy * dy + dz * dz, eps2, rs);
            }
            rows[size_t(i)] = part;
        }
    });
    double sum = 0;
    for (double r : rows) sum += r;
    return sum;
}

}  // extern "C"
