// lem_oracle.cpp -- FP64 CPU restatement of the PARALLEM per-timestep hot path.
//
// TEST INFRASTRUCTURE: the checker for the CUDA path (tests, smoke, the timed
// CPU baseline).  Each function names the reference lines it restates.  The
// reference's racy GPU sweeps are replaced by deterministic equivalents that
// reach the same fixpoints:
//   * plateau routing: the fixpoint of the float distance relaxation
//     (newflow.cu:264-350) in Dijkstra order; the final direction is the
//     first direction (N,NE,E,...) whose neighbour attains the cell's distance,
//     and the 1e-4 slope is written on that direction only;
//   * basin labels: sink ids are numbered in raster order (the reference uses
//     atomicAdd order, newflow.cu:378); merged plateaus take the largest id;
//   * boundary edges keep the exact minimum height per basin pair (the
//     reference's hash table can lose a minimum to a write race and drops
//     entries on overflow, newflow.cu:843-873);
//   * the dependency waves of correctmfdflow and sedmfdaccum are evaluated in
//     topological order (Kahn); cells that the reference never completes
//     (cycles, blocked donors) are left exactly as the reference leaves them.
// Reference behaviour that is undefined (reads outside the grid in CalcMFD /
// MFDsedbud, wrapped threads in init_watershedMFD newflow.cu:359) is not
// reproduced: out-of-grid neighbours are never donors.

#include "lem_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <queue>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// direction index d = 0..7: N, NE, E, SE, S, SW, W, NW (routeflow.cu:701-702)
const int kDx[8] = {0, 1, 1, 1, 0, -1, -1, -1};
const int kDy[8] = {-1, -1, 0, 1, 1, 1, 0, -1};
// MFD bit of direction d (newflow.cu:99-106; Directions.h:4-12)
const int kCode[8] = {64, 128, 1, 2, 4, 8, 16, 32};
const double kNoData = -9999.0;

inline float dir_dc(int d) { return (d % 2 == 0) ? 1.0f : 1.41f; }

// Index of the bit of code `c` in direction order, -1 if not a single bit.
inline int code_to_dir(int c) {
    for (int d = 0; d < 8; ++d)
        if (kCode[d] == c) return d;
    return -1;
}

// The donor scan of CalcMFD / MFDsedbud (mfd_simple.cu:95-165, mfd_accum.cu:93-221)
// visits the neighbours in the order E, SE, S, SW, W, NW, N, NE and tests the
// neighbour's code for the bit that points back at the cell.
struct DonorDir { int dx, dy, bit, slot; };
const DonorDir kDonor[8] = {
    {1, 0, 16, 6},    // east neighbour flowing west
    {1, 1, 32, 7},    // south-east neighbour flowing north-west
    {0, 1, 64, 0},    // south neighbour flowing north
    {-1, 1, 128, 1},  // south-west neighbour flowing north-east
    {-1, 0, 1, 2},    // west neighbour flowing east
    {-1, -1, 2, 3},   // north-west neighbour flowing south-east
    {0, -1, 4, 4},    // north neighbour flowing south
    {1, -1, 8, 5},    // north-east neighbour flowing south-west
};

struct Grid {
    int W, H;
    long N() const { return (long)W * H; }
    bool in(int x, int y) const { return x >= 0 && x < W && y >= 0 && y < H; }
};

// ---------------------------------------------------------------------------
// FlowDirs (FD_kernels/newflow.cu:49-174).  Writes SFD/MFD codes; when
// `slopes` is non-null the downslope slopes are stored (other entries keep
// their old values).  Returns the sink and flat counters (newflow.cu:152-164).
void flow_dirs(const Grid& g, const int32_t* mask, const double* zs, double* slopes, int32_t* sfd,
               int32_t* mfd, int cell_size, int* sinks, int* flats) {
    long sinkc = 0, flatc = 0;
#pragma omp parallel for schedule(static) reduction(+ : sinkc, flatc)
    for (int y = 0; y < g.H; ++y) {
        for (int x = 0; x < g.W; ++x) {
            long self = (long)y * g.W + x;
            mfd[self] = -9999;
            sfd[self] = -9999;
            if (mask[self] != 1) continue;
            double smax = 0.0;
            int aspect = 0, aspectsfd = 0, up = 0, flat = 0;
            for (int d = 0; d < 8; ++d) {
                int nx = x + kDx[d], ny = y + kDy[d];
                if (!g.in(nx, ny)) continue;
                double zt = zs[(long)ny * g.W + nx];
                double zc = zs[self];
                float L = (float)cell_size * dir_dc(d);
                double stemp = (zc - zt) / (double)L;
                if (zc > zt && zt != kNoData) {
                    if (slopes) slopes[8 * self + d] = stemp;
                    if (stemp > smax) {
                        smax = stemp;
                        aspectsfd = kCode[d];
                    }
                    aspect += kCode[d];
                }
                if (zc < zt) up += 1;
                if (zc == zt) flat += 1;
            }
            if (up > 7) {
                sinkc++;
                aspect = aspectsfd = 0;
            }
            if (flat + up > 7 && up <= 7) {
                flatc++;
                aspect = aspectsfd = 0;
            }
            mfd[self] = aspect;
            sfd[self] = aspectsfd;
        }
    }
    if (sinks) *sinks = (int)sinkc;
    if (flats) *flats = (int)flatc;
}

// shortest_paths_plateaus_initMFD + the route_plateausMFD loop
// (newflow.cu:234-350, routeflow.cu:826-872 and :632-642).  The reference
// sweeps dist = min(dist, dist_n + dc) over equal-height neighbours until no
// cell changes.  That relaxation is monotone, so every fair order of updates
// ends at the same fixpoint: the greatest one below the start values.  Because
// fl(d + dc) >= d for dc > 0, a Dijkstra order over the equal-height graph
// reaches it visiting every cell once: a cell popped with distance v can only
// be offered fl(v' + dc) >= v' >= v by cells popped after it.  Returns the
// number of relaxation passes (1; the reference's sweep count depends on its
// thread schedule).
int route_plateaus(const Grid& g, const int32_t* mask, const double* zs, double* slopes, int32_t* mfd,
                   int32_t* sfd, float* sp_out) {
    const long N = g.N();
    const float kFar = 20000000.0f;
    std::vector<float> sp(N, 0.0f);
    std::vector<long> cand;
    for (long i = 0; i < N; ++i) {
        if (mask[i] != 1) continue;
        sp[i] = kFar;
        if (mfd[i] > 0) sp[i] = 0;
        if (sfd[i] > 0) sp[i] = 0;
        if (sp[i] != 0) cand.push_back(i);
    }
    std::vector<char> is_cand(N, 0);
    for (long i : cand) is_cand[i] = 1;
    // seeds: every cell at distance 0 next to an equal-height candidate
    typedef std::pair<float, long> Item;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
    for (long i : cand) {
        int x = (int)(i % g.W), y = (int)(i / g.W);
        for (int d = 0; d < 8; ++d) {
            int nx = x + kDx[d], ny = y + kDy[d];
            if (!g.in(nx, ny)) continue;
            long n = (long)ny * g.W + nx;
            if (!is_cand[n] && zs[i] == zs[n]) {
                float dis = sp[n] + dir_dc(d);
                if (sp[i] > dis) {
                    sp[i] = dis;
                }
            }
        }
        if (sp[i] < kFar) heap.push(Item(sp[i], i));
    }
    while (!heap.empty()) {
        Item it = heap.top();
        heap.pop();
        long i = it.second;
        if (it.first != sp[i]) continue;  // a stale entry
        int x = (int)(i % g.W), y = (int)(i / g.W);
        for (int d = 0; d < 8; ++d) {
            int nx = x + kDx[d], ny = y + kDy[d];
            if (!g.in(nx, ny)) continue;
            long n = (long)ny * g.W + nx;
            if (!is_cand[n] || !(zs[i] == zs[n])) continue;
            float dis = sp[i] + dir_dc(d);  // the step from n to i has the same length
            if (sp[n] > dis) {
                sp[n] = dis;
                heap.push(Item(dis, n));
            }
        }
    }
    // final direction: first neighbour attaining the distance
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)cand.size(); ++k) {
        const long i = cand[k];
        if (!(sp[i] < kFar)) continue;
        int x = (int)(i % g.W), y = (int)(i / g.W);
        for (int d = 0; d < 8; ++d) {
            int nx = x + kDx[d], ny = y + kDy[d];
            if (!g.in(nx, ny)) continue;
            long n = (long)ny * g.W + nx;
            if (zs[i] == zs[n] && (float)(sp[n] + dir_dc(d)) == sp[i]) {
                mfd[i] = kCode[d];
                sfd[i] = kCode[d];
                if (slopes) slopes[8 * i + d] = 0.0001;
                break;
            }
        }
    }
    if (sp_out)
        for (long i = 0; i < N; ++i) sp_out[i] = mask[i] == 1 ? sp[i] : 0.0f;
    return cand.empty() ? 0 : 1;
}

struct UnionSet {  // union_set (newflow.cu:654-707)
    std::vector<int> parent, rank;
    explicit UnionSet(int s) : parent(s, 0), rank(s, 0) {}
    bool in_set(int x) const {
        if (x == 0) return true;
        if (x > 0 && x < (int)parent.size() && parent[x] > 0) return true;
        return false;
    }
    int find_root(int x) const {
        while (parent[x] != x) x = parent[x];
        return x;
    }
    void make_set(int x) {
        if (x > 0 && x < (int)parent.size()) {
            parent[x] = x;
            rank[x] = 0;
        }
    }
    void merge(int a, int b) {
        int ar = find_root(a), br = find_root(b);
        if (ar == br) return;
        if (rank[ar] > rank[br])
            parent[br] = ar;
        else {
            parent[ar] = br;
            if (rank[ar] == rank[br]) rank[br]++;
        }
    }
};

// floodingDriver (routeflow.cu:202-676): labels basins, computes the spill
// heights by Kruskal over the basin boundary graph and raises zs in place.
// Returns the number of distinct labels on boundary edges (data->sinkcount,
// newflow.cu:1045) and the basin labels in `ws`.
int flood(const Grid& g, const int32_t* mask, double* zs, const int32_t* sfd, std::vector<int>& ws,
          int* nbasins) {
    const long N = g.N();
    ws.assign(N, 0);
    // init_watershedMFD (newflow.cu:352-420)
    int counter = 0;
    for (int y = 0; y < g.H; ++y)
        for (int x = 0; x < g.W; ++x) {
            long i = (long)y * g.W + x;
            if (mask[i] != 1) { ws[i] = 0; continue; }
            if (x == g.W - 1 || y == 0 || y == g.H - 1) { ws[i] = 0; continue; }
            if (sfd[i] == 0) {
                ws[i] = ++counter;
            } else {
                int d = code_to_dir(sfd[i]);
                long n = (long)(y + kDy[d]) * g.W + (x + kDx[d]);
                ws[i] = -(int)(n + 1);
            }
        }
    // init_watershed_sinkMFD loop (newflow.cu:430-460, routeflow.cu:285-302):
    // equal-height sink cells adopt the largest neighbouring id until stable.
    std::vector<long> sinks;
    for (long i = 0; i < N; ++i)
        if (mask[i] == 1 && sfd[i] == 0) sinks.push_back(i);
    // The loop raises ids to the largest id over equal-height neighbours until
    // stable: a monotone relaxation, so a worklist that re-examines the
    // equal-height sink neighbours of every raised cell ends at the same
    // fixpoint (each connected run of equal-height sinks takes its largest id).
    std::vector<char> is_sink(N, 0), queued(N, 0);
    for (long i : sinks) is_sink[i] = 1;
    std::deque<long> work(sinks.begin(), sinks.end());
    for (long i : sinks) queued[i] = 1;
    while (!work.empty()) {
        long i = work.front();
        work.pop_front();
        queued[i] = 0;
        int x = (int)(i % g.W), y = (int)(i / g.W);
        int best = ws[i];
        for (int d = 0; d < 8; ++d) {
            int nx = x + kDx[d], ny = y + kDy[d];
            if (!g.in(nx, ny)) continue;
            long n = (long)ny * g.W + nx;
            if (zs[n] == zs[i] && ws[n] > best) best = ws[n];
        }
        if (best == ws[i]) continue;
        ws[i] = best;
        for (int d = 0; d < 8; ++d) {
            int nx = x + kDx[d], ny = y + kDy[d];
            if (!g.in(nx, ny)) continue;
            long n = (long)ny * g.W + nx;
            if (is_sink[n] && !queued[n] && zs[n] == zs[i] && ws[n] < best) {
                queued[n] = 1;
                work.push_back(n);
            }
        }
    }
    // identify_watershedMFD loop (newflow.cu:469-487, routeflow.cu:314-338)
    for (long i = 0; i < N; ++i) {
        if (mask[i] != 1 || ws[i] >= 0) continue;
        std::vector<long> path;
        long c = i;
        while (ws[c] < 0) {
            path.push_back(c);
            c = -(long)ws[c] - 1;
            if ((long)path.size() > N) break;  // cycle guard (cannot happen: sfd descends)
        }
        int lab = ws[c] < 0 ? 0 : ws[c];
        for (long p : path) ws[p] = lab;
    }
    // identify_watershed_boundary_write_backMFD (newflow.cu:787-877): for every
    // pair of neighbouring cells with different labels the higher cell gives a
    // boundary height; the minimum per unordered label pair is kept.
    struct Pair { int a, b; double w; };
    std::vector<Pair> pairs;
#pragma omp parallel
    {
        std::vector<Pair> mine;
#pragma omp for schedule(static)
        for (int y = 0; y < g.H; ++y)
            for (int x = 0; x < g.W; ++x) {
                long i = (long)y * g.W + x;
                if (mask[i] != 1) continue;
                int a = ws[i];
                for (int d = 0; d < 8; ++d) {
                    int nx = x + kDx[d], ny = y + kDy[d];
                    if (!g.in(nx, ny)) continue;
                    long n = (long)ny * g.W + nx;
                    int b = ws[n];
                    if (a == b) continue;
                    if (!(zs[i] >= zs[n])) continue;
                    mine.push_back({std::min(a, b), std::max(a, b), zs[i]});
                }
            }
#pragma omp critical
        pairs.insert(pairs.end(), mine.begin(), mine.end());
    }
    // the minimum height per unordered label pair, pairs in ascending order
    std::sort(pairs.begin(), pairs.end(), [](const Pair& p, const Pair& q) {
        return p.a != q.a ? p.a < q.a : p.b != q.b ? p.b < q.b : p.w < q.w;
    });
    std::vector<std::pair<std::pair<int, int>, double>> edges;
    for (size_t k = 0; k < pairs.size(); ++k)
        if (k == 0 || pairs[k].a != pairs[k - 1].a || pairs[k].b != pairs[k - 1].b)
            edges.push_back({{pairs[k].a, pairs[k].b}, pairs[k].w});
    // init_and_sort_watershed_bound_labelsMFD (newflow.cu:905-1050) + Kruskal
    // (routeflow.cu:510-572)
    struct E { int a, b; double w; };
    std::vector<E> list;
    list.reserve(edges.size());
    int max_label = 0;
    std::vector<int> seen;
    for (auto& kv : edges) {
        list.push_back({kv.first.first, kv.first.second, kv.second});
        max_label = std::max(max_label, kv.first.second);
        seen.push_back(kv.first.first);
        seen.push_back(kv.first.second);
    }
    std::sort(seen.begin(), seen.end());
    int distinct = (int)(std::unique(seen.begin(), seen.end()) - seen.begin());
    std::stable_sort(list.begin(), list.end(), [](const E& p, const E& q) { return p.w < q.w; });
    UnionSet set(max_label + 1);
    std::vector<char> done(max_label + 1, 0);
    std::vector<double> raise(max_label + 1, 0.0);
    done[0] = 1;
    for (const E& e : list) {
        if (!set.in_set(e.a)) set.make_set(e.a);
        if (!set.in_set(e.b)) set.make_set(e.b);
        int r1 = set.find_root(e.a), r2 = set.find_root(e.b);
        if (done[r1] && done[r2]) continue;
        if (done[r1] || done[r2]) {
            if (done[r1]) { done[r2] = 1; raise[r2] = e.w; }
            else { done[r1] = 1; raise[r1] = e.w; }
            continue;
        }
        if (r1 != r2) {
            set.merge(r1, r2);
            raise[r2] = raise[r1] = e.w;
        }
    }
    for (int i = 0; i <= max_label; ++i)
        if (raise[i] != 0) raise[i] = raise[set.find_root(i)];
    // raise_watershedMFD (newflow.cu:879-894)
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) {
        if (mask[i] != 1) continue;
        int lab = ws[i];
        double r = (lab >= 0 && lab <= max_label) ? raise[lab] : 0.0;
        if (zs[i] < r) zs[i] = r;
    }
    int basins = 0;
    for (int i = 1; i <= max_label; ++i)
        if (set.in_set(i)) ++basins;
    if (nbasins) *nbasins = basins;
    return distinct;
}

// Dependency-wave evaluation shared by correctmfdflow and sedmfdaccum.
// A cell is processed once all its donors are done; `processable` cells
// become done when processed, `done0` cells are done from the start, all
// other cells never become done.  `visit` is called in a topological order.
template <class Visit>
long wave(const Grid& g, const int32_t* fd, const std::vector<char>& processable,
          const std::vector<char>& done0, Visit visit) {
    const long N = g.N();
    std::vector<int> pending(N, 0);
    std::vector<char> blocked(N, 0);
    for (int y = 0; y < g.H; ++y)
        for (int x = 0; x < g.W; ++x) {
            long c = (long)y * g.W + x;
            if (!processable[c]) continue;
            for (int k = 0; k < 8; ++k) {
                int nx = x + kDonor[k].dx, ny = y + kDonor[k].dy;
                if (!g.in(nx, ny)) continue;
                long n = (long)ny * g.W + nx;
                if (!(fd[n] & kDonor[k].bit)) continue;
                if (processable[n]) pending[c]++;
                else if (!done0[n]) blocked[c] = 1;
            }
        }
    std::deque<long> q;
    for (long c = 0; c < N; ++c)
        if (processable[c] && !blocked[c] && pending[c] == 0) q.push_back(c);
    long ndone = 0;
    while (!q.empty()) {
        long c = q.front();
        q.pop_front();
        visit(c);
        ++ndone;
        int x = (int)(c % g.W), y = (int)(c / g.W);
        // receivers: neighbours r for which c is a donor
        for (int k = 0; k < 8; ++k) {
            int rx = x - kDonor[k].dx, ry = y - kDonor[k].dy;
            if (!g.in(rx, ry)) continue;
            if (!(fd[c] & kDonor[k].bit)) continue;
            long r = (long)ry * g.W + rx;
            if (!processable[r]) continue;
            if (--pending[r] == 0 && !blocked[r]) q.push_back(r);
        }
    }
    return ndone;
}

}  // namespace

extern "C" {

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void oracle_set_climate(oracle_state* s, int init) {
    // SetClimateMatrices (MEM_kernels/Data.cpp:211-303)
    const int W = s->W, H = s->H;
    if (init) {
        s->last_rain = s->rain;
        s->last_temp = s->temp;
    }
    const double minheight = 467.228;
    double rainmax = s->rain * 2, rainmin = s->rain;
    double increment = (rainmax - rainmin) / H;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H; ++i) {
        double therain = rainmin + (i * increment);
        for (int j = 0; j < W; ++j) {
            long c = (long)i * W + j;
            if (s->mask[c] == 1) {
                s->rainmat[c] = therain;
                s->tempmat[c] = s->temp - ((s->dem[c] - minheight) * 0.0065);
            } else {
                s->rainmat[c] = -9999.;
                s->tempmat[c] = -9999.;
            }
        }
    }
    if (init) {
        double Lrainmax = s->last_rain * 2, Lrainmin = s->last_rain;
        double Linc = (Lrainmax - Lrainmin) / H;
#pragma omp parallel for schedule(static)
        for (int i = 0; i < H; ++i) {
            double therain = Lrainmin + (i * Linc);
            for (int j = 0; j < W; ++j) {
                long c = (long)i * W + j;
                if (s->mask[c] == 1) {
                    s->last_rainmat[c] = therain;
                    s->last_tempmat[c] = s->last_temp - ((s->dem[c] - minheight) * 0.0065);
                } else {
                    s->last_rainmat[c] = -9999.;
                    s->last_tempmat[c] = -9999.;
                }
            }
        }
    }
}

void oracle_init_mask_outlet(oracle_state* s) {
    const long N = (long)s->W * s->H;
    // createmask (MEM_kernels/memory.cu:229-238)
    for (long x = 0; x < N; ++x) s->mask[x] = (s->dem[x] == -9999) ? 0 : 1;
    // init_setoutletcell (MEM_kernels/Data.cpp:38-66)
    double lowest = 1000.;
    int index = 0;
    for (long c = 0; c < N; ++c)
        if (s->mask[c] == 1 && s->dem[c] < lowest) {
            lowest = s->dem[c];
            index = (int)c;
        }
    s->outlet = index;
}

void oracle_init_process(oracle_state* s, double stoneval, double fineval, double soilMval,
                         double nutval, double soilBval) {
    // setProcessMatrices (MEM_kernels/Data.cpp:115-209).  soilT is left as set
    // by the caller (createSoilTfromformula or a raster in the reference).
    const long N = (long)s->W * s->H;
    double rescale = (10000 / (s->cellsize * s->cellsize));
    for (long x = 0; x < N; ++x) {
        s->fd[x] = 0;
        s->sfd[x] = 0;
        s->fa[x] = 0.0;
        s->slopeptr[x] = 0.0;
        s->dz[x] = 0.0;
        if (s->mask[x] == 1) {
            s->runoff[x] = 1.0;
            s->stone[x] = stoneval;
            s->fines[x] = fineval;
            s->soilM[x] = soilMval;
            s->nut[x] = nutval;
            s->soilB[x] = soilBval;
            double tempeffect = 100 + (100 / (s->tempmat[x] + 15));
            s->totB[x] = (3000.0 + (5.0 * (s->rainmat[x] - tempeffect))) / rescale;
        } else {
            s->runoff[x] = 0.0;
            s->soilT[x] = 0.0;
            s->stone[x] = s->fines[x] = s->soilM[x] = s->nut[x] = s->soilB[x] = s->totB[x] = 0.0;
        }
        s->ero[x] = s->geli[x] = s->inci[x] = s->depo[x] = s->wC[x] = s->wP[x] = 0.0;
    }
    for (long y = 0; y < 8 * N; ++y) {
        s->slopes[y] = 0.0;
        s->prop[y] = 0.0;
    }
}

int oracle_flow_direction(oracle_state* s, const lem_params* p) {
    Grid g{s->W, s->H};
    const long N = g.N();
    const int csize = (int)s->cellsize;
    // device copy of the DEM (routeflow.cu:731); the host outlet adjustment of
    // routeflow.cu:740-741 happens after the copy and so is not seen here.
    std::vector<double> zd(s->dem, s->dem + N);
    double lowest = 1000.;
    for (long x = 0; x < N; ++x)
        if (s->mask[x] == 1 && s->dem[x] < lowest) lowest = s->dem[x];
    if (lowest < s->dem[s->outlet]) s->dem[s->outlet] = lowest - 0.0001;

    std::vector<int32_t> mfd(N), sfd(N);
    int sinks = 0, flats = 0;
    flow_dirs(g, s->mask, zd.data(), s->slopes, sfd.data(), mfd.data(), csize, &sinks, &flats);
    s->init_sinks = sinks;
    s->init_flats = flats;
    int sweeps = route_plateaus(g, s->mask, zd.data(), s->slopes, mfd.data(), sfd.data(), s->shortest_paths);
    if (s->sfd_pass1)
        for (long j = 0; j < N; ++j) s->sfd_pass1[j] = sfd[j];
    // routeflow.cu:893-909: sinks left after plateau routing
    int sinkcount = 0;
    for (long j = 0; j < N; ++j)
        if (s->mask[j] == 1 && sfd[j] == 0) sinkcount++;
    s->sinkcount = sinkcount;
    s->flood_basins = 0;
    if (s->watershed)
        for (long j = 0; j < N; ++j) s->watershed[j] = 0;
    if (sinkcount > 0) {
        std::vector<int> ws;
        int basins = 0;
        s->sinkcount = flood(g, s->mask, zd.data(), sfd.data(), ws, &basins);
        s->flood_basins = basins;
        if (s->watershed)
            for (long j = 0; j < N; ++j) s->watershed[j] = ws[j];
        // second FlowDirs and plateau pass on the raised DEM (routeflow.cu:623-642);
        // their slopes never reach the host copy, so they are not stored.
        flow_dirs(g, s->mask, zd.data(), nullptr, sfd.data(), mfd.data(), csize, nullptr, nullptr);
        sweeps += route_plateaus(g, s->mask, zd.data(), nullptr, mfd.data(), sfd.data(), s->shortest_paths);
    }
    s->plateau_sweeps = sweeps;
    if (s->dem_routed)
        for (long i = 0; i < N; ++i) s->dem_routed[i] = zd[i];
    // epilogue (routeflow.cu:934-953)
    for (long i = 0; i < N; ++i) {
        s->sfd[i] = sfd[i];
        s->fd[i] = mfd[i];
    }
    if (p->flow_direction_type == 0) {
        for (long i = 0; i < N; ++i) s->fd[i] = s->sfd[i];
    } else {
        for (long i = 0; i < N; ++i)
            if (s->fd[i] <= 0 && s->mask[i] == 1) s->fd[i] = s->sfd[i];
    }
    s->fd[s->outlet] = 16;
    return 0;
}

static void calc_props(oracle_state* s) {
    // calcprops (MOD_kernels/runoffweight.cu:141-354)
    const long N = (long)s->W * s->H;
    for (long i = 0; i < N; ++i) {
        if (s->mask[i] != 1) continue;
        long si = i * 8;
        double slopetot = 0;
        for (int k = 0; k < 8; ++k) slopetot += s->slopes[si + k];
        int propdircount = 0;
        for (int k = 0; k < 8; ++k) {
            s->prop[si + k] = s->slopes[si + k] / slopetot;
            if (s->prop[si + k] > 0) propdircount++;
        }
        int d = code_to_dir(s->fd[i]);
        if (d >= 0 && propdircount > 1) {
            for (int z = 0; z < 8; ++z) {
                s->slopes[si + z] = (z == d) ? 0.0001 : 0.0;
                s->prop[si + z] = (z == d) ? 1.0 : 0.0;
            }
        }
    }
}

int oracle_flow_accumulation(oracle_state* s, const lem_params* p, uint32_t flags) {
    Grid g{s->W, s->H};
    const long N = g.N();
    // calcrunoffweight (MOD_kernels/runoffweight.cu:21-58)
#pragma omp parallel for schedule(static)
    for (long c = 0; c < N; ++c) {
        if (s->mask[c] == 0) {
            s->runoff[c] = -9999;
            continue;
        }
        double coeff = (1.0 - 0.0085 * (s->stone[c])) * exp(-0.0025 * (s->totB[c]) / 76.5) *
                       tanh(0.6 + (s->soilM[c]) / 0.2);
        double myppt = s->rainmat[c] / 1000;
        s->runoff[c] = myppt * coeff;
        s->soilM[c] += myppt * (1. - coeff);
        if (s->soilM[c] > 0.5) s->soilM[c] = 0.5;
    }
    // calcpropsSFD (runoffweight.cu:115-138) or calcprops (:141-354)
    if (p->flow_direction_type != 0 && p->mfd_proportions) {
        calc_props(s);
    } else {
        for (long i = 0; i < N; ++i)
            for (int k = 0; k < 8; ++k) s->prop[i * 8 + k] = (s->mask[i] == 1) ? 1.0 : 0.0;
    }
    // correctmfdflow (FA_kernels/mfd_simple.cu:238-305) evaluated as its fixpoint
    std::vector<char> processable(N), done0(N);
    for (long c = 0; c < N; ++c) {
        processable[c] = s->mask[c] == 1;
        done0[c] = s->dem[c] == -9999;
        s->fa[c] = processable[c] ? s->runoff[c] : 0.0;  // CalcMFD writes fa = w first (:72)
    }
    long ndone = wave(g, s->fd, processable, done0, [&](long c) {
        int x = (int)(c % g.W), y = (int)(c / g.W);
        double accum = 0.;
        for (int k = 0; k < 8; ++k) {
            int nx = x + kDonor[k].dx, ny = y + kDonor[k].dy;
            if (!g.in(nx, ny)) continue;
            long n = (long)ny * g.W + nx;
            if (!(s->fd[n] & kDonor[k].bit)) continue;
            accum += s->fa[n] * s->prop[n * 8 + kDonor[k].slot];
        }
        if (accum < 0.0) accum = 0.0;
        s->fa[c] = s->runoff[c] + accum;
    });
    long active = 0;
    for (long c = 0; c < N; ++c) active += s->mask[c] != 0;
    s->fa_uncomputed = (int)(active - ndone);
    if (s->contrib) {
        for (long c = 0; c < N; ++c) s->contrib[c] = processable[c] ? 1 : 0;
        wave(g, s->fd, processable, done0, [&](long c) {
            int x = (int)(c % g.W), y = (int)(c / g.W);
            int32_t acc = 1;
            for (int k = 0; k < 8; ++k) {
                int nx = x + kDonor[k].dx, ny = y + kDonor[k].dy;
                if (!g.in(nx, ny)) continue;
                long n = (long)ny * g.W + nx;
                if ((s->fd[n] & kDonor[k].bit) && processable[n]) acc += s->contrib[n];
            }
            s->contrib[c] = acc;
        });
    }
    // FA_max / outlet (mfd_simple.cu:332-357)
    if (flags & LEM_STEP_SET_OUTLET_FROM_FA) {
        double m = 0.0;
        int idx = 0;
        for (long i = 0; i < N; ++i)
            if (s->fa[i] > m) {
                m = s->fa[i];
                idx = (int)i;
            }
        s->FA_max = m;
        s->outlet = idx;
    } else {
        double m = 0.0;
        for (long i = 0; i < N; ++i) m = std::max(m, s->fa[i]);
        s->FA_max = m;
    }
    return 0;
}

int oracle_erosion(oracle_state* s, lem_params* p) {
    Grid g{s->W, s->H};
    const long N = g.N();
    const double cs = s->cellsize;
    // aveslope (MOD_kernels/eroincidep.cu:8-37)
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) {
        s->slopeptr[i] = 0.0;
        if (s->mask[i] == 1) {
            double total = 0;
            int nonzero = 0;
            for (int j = 0; j < 8; ++j) {
                total += s->slopes[i * 8 + j];
                if (s->slopes[i * 8 + j] > 0) nonzero++;
            }
            if (total > 0 && nonzero > 0) s->slopeptr[i] = total / nonzero;
        }
    }
    // diff_erosion, conc_erosion, gelifluction (eroincidep.cu:39-198)
    const double rescale_c = 1 / (10000 / (cs * cs));
#pragma omp parallel for schedule(static)
    for (long c = 0; c < N; ++c) {
        if (s->mask[c] == 0) {
            s->ero[c] = s->inci[c] = s->geli[c] = 0.0;
            continue;
        }
        double erodibility = (2.77e-6 * pow(s->fines[c], 1.14) * (12. - s->nut[c])) +
                             (0.043 * (p->soil_struct - 2.)) + (0.033 * (p->profile_permeability - 3.));
        if (erodibility < 0.0) erodibility = 0.0;
        double OF = ((s->fa[c]) * 1000) / 25;
        if (OF > p->q_threshold) OF = p->q_threshold;
        double slope = s->slopeptr[c];
        if (slope == 0.0) slope = 0.0001;
        if (slope > 5.0) slope = 5.0;
        double answer = ((erodibility * OF * OF * pow(slope, 1.67) * (pow((110. - (s->stone[c])), 0.877) / 61.7023))) *
                        exp(-0.07 * (s->totB[c]) / 76.5);
        if (answer > s->soilT[c]) answer = s->soilT[c];
        s->ero[c] = answer;

        double cslope = s->slopeptr[c];
        if (cslope > 0.5) cslope = 0.5;
        double f_temp = ((s->fa[c]) * rescale_c) - p->q_threshold;
        double inci;
        if (f_temp < 0.0) {
            f_temp = 0.0;
            inci = 0.0;
        } else {
            if (cslope == 0.0)
                inci = p->flow_a * pow(f_temp, p->flow_b) * 0.01 * exp(-0.07 * (s->totB[c]) / 76.5);
            else
                inci = p->flow_a * pow(f_temp, p->flow_b) * (cslope) * exp(-0.07 * (s->totB[c]) / 76.5);
        }
        if (inci > p->max_incision) inci = p->max_incision;
        if (inci > s->soilT[c]) {
            double softrockinc = s->soilT[c];
            double bedrockinc = (1.0 - (softrockinc / inci)) * 0.0001 * pow(f_temp, p->flow_b) * (cslope) *
                                exp(-0.07 * (s->totB[c]) / 76.5);
            inci = softrockinc + bedrockinc;
            if (inci > p->max_incision) inci = p->max_incision;
        }
        s->inci[c] = inci;

        double T = s->tempmat[c];
        double kappa = p->kappa;
        if (T >= -20. && T <= 8.87)
            kappa = 0.15711 - 0.011835 * T - 0.001195 * T * T + 0.000038 * T * T * T + 0.000002 * T * T * T * T;
        double scaler = 1 - (s->fa[c] / p->g_flowlim);
        if (s->fa[c] > p->g_flowlim) scaler = 0.0;
        double slopethreshold = s->slopeptr[c];
        if (slopethreshold > p->g_slope) slopethreshold = p->g_slope;
        double geli = kappa * slopethreshold * scaler;
        if ((s->ero[c] + geli) > s->soilT[c]) geli = s->soilT[c] - s->ero[c];
        if (geli < 0.0) geli = 0.0;
        s->geli[c] = geli;
    }
    double totE = 0, totI = 0, totG = 0;
    for (long c = 0; c < N; ++c) {
        totE += s->ero[c];
        totI += s->inci[c];
        totG += s->geli[c];
    }
    s->totE = totE;
    s->totI = totI;
    s->totG = totG;

    // sedmfdaccum (MOD_kernels/mfd_accum.cu:345-483) with MFDsedbud (:32-254)
    if (p->ddk > 0.95) p->ddk = 0.95;
    if (p->dck > 0.9) p->dck = 0.9;
    const double ddk = p->ddk, dck = p->dck, dgk = p->dgk;
    for (long x = 0; x < N; ++x)
        if (s->mask[x] == 1) s->depo[x] = 0.00001;
    std::vector<char> processable(N), done0(N, 0);
    for (long c = 0; c < N; ++c) {
        int x = (int)(c % g.W), y = (int)(c / g.W);
        processable[c] = (s->mask[c] != 0) && x != 0 && y != 0;
    }
    long ndone = wave(g, s->fd, processable, done0, [&](long c) {
        int x = (int)(c % g.W), y = (int)(c / g.W);
        double accum_d = 0.0, accum_c = 0.0, accum_g = 0.0;
        double from[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 8; ++k) {
            int nx = x + kDonor[k].dx, ny = y + kDonor[k].dy;
            if (!g.in(nx, ny)) continue;
            long n = (long)ny * g.W + nx;
            if (!(s->fd[n] & kDonor[k].bit)) continue;
            double pr = s->prop[n * 8 + kDonor[k].slot];
            accum_d += pr * (s->ero[n] * (1 - ddk));
            accum_c += pr * (s->inci[n] * (1 - dck));
            accum_g += pr * (s->geli[n] * (1 - dgk));
            from[k] = pr * s->stone[n];
        }
        s->depo[c] = ((accum_d + s->ero[c]) * ddk) + ((accum_c + s->inci[c]) * dck) + ((accum_g + s->geli[c]) * dgk);
        double sedthick = (s->soilT[c]) + (s->depo[c]);
        if (sedthick != 0.0) {
            double old = (s->soilT[c]) / sedthick;
            double input = 1 - old;
            double propStonefrom = (from[0] + from[1] + from[2] + from[3] + from[4] + from[5] + from[6] + from[7]);
            s->stone[c] = (old * (s->stone[c])) + (input * (propStonefrom));
            if (s->stone[c] < 0.01)
                s->stone[c] = 0.01;
            else if (s->stone[c] > 99.9)
                s->stone[c] = 99.9;
            s->fines[c] = 100 - s->stone[c];
        }
        double toterosion = s->ero[c] + s->inci[c] + s->geli[c];
        if (toterosion >= sedthick) s->soilT[c] = 0.0;
        if (sedthick > toterosion) s->soilT[c] = sedthick - toterosion;
    });
    long active = 0;
    for (long c = 0; c < N; ++c) active += s->mask[c] != 0;
    s->sed_uncomputed = (int)(active - ndone);
    double totD = 0;
    for (long c = 0; c < N; ++c) totD += s->depo[c];
    s->totD = totD;

    // surface_change (eroincidep.cu:200-217) and weathering (:220-327, type 1)
    const double rescale_w = 10000 * (10000 / (cs * cs));
#pragma omp parallel for schedule(static)
    for (long c = 0; c < N; ++c) {
        if (s->mask[c] == 0) {
            s->dz[c] = 0.0;
            s->wP[c] = 0.0;
            s->wC[c] = 0.0;
            continue;
        }
        s->dz[c] = (s->depo[c] - s->ero[c] - s->inci[c] - s->geli[c]);
        double T = s->tempmat[c];
        double PE_d = 1.44 * pow(T + 6., 2);
        double P0_d = 7.7e-5, P1_d = 2.3;
        double t_abs = T + 273.16;
        double t2 = t_abs * t_abs;
        double ltemp = log10(t_abs);
        double DHA = -0.4883 + 8.074e-4 * T;
        double DHB = -0.3241 + 1.600e-4 * T;
        double sqI = sqrt(0.1);
        double denom1 = (-4. * DHA * sqI) / (1. + 5.e-8 * DHB * sqI);
        double gammCa_d = pow(10., denom1);
        double gammHCO3_d = pow(10., (-DHA * sqI) / (1. + 5.4e-8 * DHB * sqI));
        double K1_d = pow(10., -356.3094 - 0.06091964 * t_abs + 21834.37 / t_abs + 126.8339 * ltemp - 1684915 / t2);
        double K2_d = pow(10., -107.8871 - 0.03252849 * t_abs + 5151.79 / t_abs + 38.92561 * ltemp - 563713.9 / t2);
        double KC_d = pow(10., -171.9065 - 0.077993 * t_abs + 2839.319 / t_abs + 71.595 * ltemp);
        double KH_d = pow(10., 108.3865 + 0.01985076 * t_abs - 6919.53 / t_abs - 40.45154 * ltemp + 669365.0 / t2);
        double surface_flow = s->fa[c] * 1000;
        double evap_trans;
        if (s->rainmat[c] + surface_flow <= PE_d)
            evap_trans = s->rainmat[c] + surface_flow;
        else
            evap_trans = s->rainmat[c] + surface_flow - PE_d;
        double PCO2;
        if (s->soilT[c] > 0.1)
            PCO2 = pow(10., -2.5 + ((T - 15.) / 10.));
        else
            PCO2 = pow(10., -3.5 + ((T - 15.) / 10.));
        double Ca2eq = pow(PCO2 * ((K1_d * KC_d * KH_d) / (4. * K2_d * gammCa_d * gammHCO3_d * gammHCO3_d)), (1. / 3.));
        double wC = 0.0148148148 * Ca2eq * (surface_flow / rescale_w);
        if (wC <= 0.0) wC = 0.0;
        if (wC > 0.001) wC = 0.001;
        double wP = P0_d * exp(-(P1_d)*s->soilT[c]);
        s->wC[c] = wC;
        s->wP[c] = wP;
        s->soilT[c] = s->soilT[c] + wC * 0.02 + wP;
        if (s->soilT[c] <= 0.0) {
            s->soilT[c] = 0.0;
            s->stone[c] = 0.0;
            s->fines[c] = 0.0;
            s->soilM[c] = 0.02;
        } else {
            if (wP > 0)
                s->stone[c] += s->stone[c] * (tanh(((s->ero[c] / s->soilT[c]))) * -tanh(((wC / wP))));
            else
                s->stone[c] += s->stone[c] * tanh(((s->ero[c] / s->soilT[c])));
            if (s->stone[c] < 0.01)
                s->stone[c] = 0.01;
            else if (s->stone[c] > 99.9)
                s->stone[c] = 99.9;
            s->fines[c] = 100. - s->stone[c];
            s->soilM[c] -= (1.e-3 * evap_trans / s->soilT[c]);
            if (s->soilM[c] < 0.02)
                s->soilM[c] = 0.02;
            else if (s->soilM[c] > 0.5)
                s->soilM[c] = 0.5;
        }
    }
    double totWC = 0, totWP = 0;
    for (long c = 0; c < N; ++c) {
        totWC += s->wC[c];
        totWP += s->wP[c];
    }
    s->totWC = totWC;
    s->totWP = totWP;

    // update_newSurface (MOD_kernels/updates.cu:142-181) with Update_Surface (:23-46)
    double base_level = s->dem[s->outlet] - 0.00012;
#pragma omp parallel for schedule(static)
    for (long c = 0; c < N; ++c) {
        if (s->mask[c] == 0) continue;
        s->dem[c] = s->dem[c] + s->dz[c] - s->wC[c] - s->wP[c];
        if (s->dem[c] <= base_level) s->dem[c] = base_level + 0.01;
    }
    s->dem[s->outlet] = base_level;
    s->dem[s->outlet] = s->dem[s->outlet] - 0.00012;

    // update_nutrient_content (updates.cu:48-76) and grow_vegetation (:78-139)
    const double rescale_v = (10000 / (cs * cs));
#pragma omp parallel for schedule(static)
    for (long c = 0; c < N; ++c) {
        if (s->mask[c] == 0) {
            s->totB[c] = 0;
            continue;
        }
        double T = s->tempmat[c];
        if (s->soilT[c] <= 0.0) s->nut[c] = 0.0;
        double leaf_fall = s->totB[c] / (72.8 * log(s->totB[c] + 1.4));
        double decomposition = s->soilB[c] * exp(0.12 * T - 5.75);
        s->soilB[c] = s->soilB[c] + leaf_fall - decomposition;
        if (s->soilT[c] == 0.0 && s->soilB[c] > 0.0)
            s->nut[c] = 100.0;
        else if (s->soilT[c] == 0.0)
            s->nut[c] = 0.0;
        else
            s->nut[c] = (s->soilB[c] / (1300. * s->soilT[c])) * 100.;
        if (s->nut[c] > 100) s->nut[c] = 100.;

        double delta_temp = T - s->last_tempmat[c];
        double tempeffect = 100 + (100 / (T + 15));
        double total_cc = (3000.0 + (5.0 * (s->rainmat[c] - tempeffect))) / rescale_v;
        if (delta_temp > 0) {
            double r_plus = delta_temp * (1.0 + tanh((T - p->temp_inflex) / p->temp_sens));
            s->totB[c] += ((r_plus * s->totB[c]) * (1. - (s->totB[c] / total_cc)));
        }
        if (delta_temp < 0) {
            double r_minus = delta_temp * (1.0 - tanh((T - p->temp_inflex) / p->temp_sens));
            s->totB[c] += ((r_minus * s->totB[c]) * (s->totB[c] / total_cc));
        }
        if (delta_temp == 0) s->totB[c] = total_cc;
        if (s->totB[c] < 1) s->totB[c] = 1.0;
    }
    double totbio = 0;
    for (long c = 0; c < N; ++c) totbio += s->totB[c];
    s->totbio = totbio;
    return 0;
}

int oracle_step(oracle_state* s, lem_params* p, const lem_climate* c, uint32_t flags) {
    if (c && c->recompute) {
        s->last_rain = s->rain;
        s->last_temp = s->temp;
        s->rain = c->rain;
        s->temp = c->temp;
        oracle_set_climate(s, 0);
    }
    oracle_flow_direction(s, p);
    oracle_flow_accumulation(s, p, flags);
    oracle_erosion(s, p);
    return 0;
}

}  // extern "C"
