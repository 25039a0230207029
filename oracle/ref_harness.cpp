// ref_harness.cpp -- runs the reference's own kernels (copied out of its
// sources at build time into _ref/ref_kernels.inc, see ref_build.py) on the CPU
// with the host loops of cuFlowDirection / floodingDriver (routeflow.cu:202-975),
// correctmfdflow (mfd_simple.cu:174-384) and erosionGPU / sedmfdaccum /
// update_newSurface (erosion.cu:69-186, mfd_accum.cu:256-483, updates.cu:142-225).
//
// TEST INFRASTRUCTURE: a second checker of the oracle.  Kernels run as one
// sequential schedule (ref_shim.h).  Every array gets spare room past its end
// because some reference threads index past the grid (init_watershedMFD only
// checks the row, newflow.cu:359; init_hash_tableMFD writes one row and column
// past its table, newflow.cu:740).
#include <vector>

#include "config.h"
#include "Directions.h"
#include "production.h"
#include "lem_oracle.h"

// calcprops reads these members of the host Data struct
struct DataProps {
    struct {
        int width, height;
    } mapInfo;
    int* mask;
    double* Slopes;
    double* prop;
    int* fd;
};

#include "ref_kernels.inc"

namespace {

int kXmove[9] = {0, 1, 1, 1, 0, -1, -1, -1, 0};
int kYmove[9] = {-1, -1, 0, 1, 1, 1, 0, -1, 0};
const int kTableSize = 30000;  // routeflow.cu:375-376
const int kListSize = 800;

template <class T>
std::vector<T> pad_copy(const T* src, size_t n, size_t extra, T fill) {
    std::vector<T> v(n + extra, fill);
    if (src) std::copy(src, src + n, v.begin());
    return v;
}

struct G {
    int W, H;
    size_t N, pad;
    dim3 grid, block;
};
G geom(const oracle_state* s) {
    G g;
    g.W = s->W;
    g.H = s->H;
    g.N = (size_t)s->W * s->H;
    g.pad = 2 * (size_t)s->W + 1024;
    g.grid = dim3(s->W / 16 + 1, s->H / 16 + 1);
    g.block = dim3(16, 16);
    return g;
}

void plateau_loop(const G& g, std::vector<int>& mask, std::vector<double>& dem, std::vector<double>& slopes,
                  std::vector<int>& fd, std::vector<int>& sfd, std::vector<float>& sp, std::vector<double>& low,
                  int csize, int* sweeps) {
    ref_launch(g.grid, g.block, shortest_paths_plateaus_initMFD, mask.data(), dem.data(), fd.data(), sfd.data(),
               sp.data(), csize, g.W, g.H, low.data());
    int flag;
    do {
        flag = 0;
        ref_launch(g.grid, g.block, route_plateausMFD, mask.data(), dem.data(), slopes.data(), fd.data(), sfd.data(),
                   sp.data(), g.W, g.H, kXmove, kYmove, &flag, low.data());
        ++*sweeps;
    } while (flag && *sweeps < 10000000);
}

}  // namespace

extern "C" {

int ref_flow_direction(oracle_state* s, const lem_params* p) {
    const G g = geom(s);
    const int csize = (int)s->cellsize;
    std::vector<int> mask = pad_copy(s->mask, g.N, g.pad, 0);
    std::vector<int> flatmask(g.N + g.pad, 0);
    std::vector<double> dem = pad_copy(s->dem, g.N, g.pad, -9999.0);  // device copy (routeflow.cu:731)
    double lowest = 1000.;                                            // testoutletislowest (:171-184)
    for (size_t x = 0; x < g.N; ++x)
        if (s->mask[x] == 1 && s->dem[x] < lowest) lowest = s->dem[x];
    if (lowest < s->dem[s->outlet]) s->dem[s->outlet] = lowest - 0.0001;
    std::vector<double> slopes = pad_copy(s->slopes, 8 * g.N, 8 * g.pad, 0.0);
    std::vector<int> fd(g.N + g.pad, 0), sfd(g.N + g.pad, 0), ws(g.N + g.pad, 0);
    std::vector<float> sp(g.N + g.pad, 0.f);
    std::vector<double> low(g.N + g.pad, 0.0);
    int sinkc = 0, flatc = 0;
    ref_launch(g.grid, g.block, FlowDirs, mask.data(), flatmask.data(), dem.data(), slopes.data(), sfd.data(),
               fd.data(), 1, csize, g.W, g.H, kXmove, kYmove, 0, &sinkc, &flatc);
    s->init_sinks = sinkc;
    s->init_flats = flatc;
    int sweeps = 0;
    plateau_loop(g, mask, dem, slopes, fd, sfd, sp, low, csize, &sweeps);
    std::copy(slopes.begin(), slopes.begin() + 8 * g.N, s->slopes);  // routeflow.cu:883
    if (s->sfd_pass1) std::copy(sfd.begin(), sfd.begin() + g.N, s->sfd_pass1);
    int sinkcount = 0;
    for (size_t j = 0; j < g.N; ++j)
        if (mask[j] == 1 && sfd[j] == 0) sinkcount++;
    s->sinkcount = sinkcount;
    if (sinkcount > 0) {
        // floodingDriver (routeflow.cu:202-676)
        int counter = 0, flag;
        ref_launch(g.grid, g.block, init_watershedMFD, mask.data(), sfd.data(), ws.data(), dem.data(), sp.data(),
                   kXmove, kYmove, &counter, g.W, g.H);
        do {
            flag = 0;
            ref_launch(g.grid, g.block, init_watershed_sinkMFD, mask.data(), sfd.data(), ws.data(), dem.data(), kXmove,
                       kYmove, g.W, g.H, &flag);
        } while (flag);
        do {
            flag = 0;
            ref_launch(g.grid, g.block, identify_watershedMFD, mask.data(), sfd.data(), ws.data(), kXmove, kYmove, g.W,
                       g.H, &flag);
        } while (flag);
        std::vector<double> hash((size_t)(kTableSize + 2) * (kListSize + 2) * 3, 0.0);
        std::vector<int> table_counter(kTableSize + 2, 0);
        ref_launch(dim3(kListSize / 16 + 1, kTableSize / 16 + 1), dim3(16, 16), init_hash_tableMFD, hash.data(),
                   table_counter.data(), kTableSize, kListSize);
        int is_succeeded = 1;
        ref_launch(g.grid, g.block, identify_watershed_boundary_write_backMFD, mask.data(), ws.data(), dem.data(),
                   hash.data(), table_counter.data(), kTableSize, kListSize, kXmove, kYmove, g.W, g.H, &is_succeeded,
                   &counter);
        int sorted_list_size = 0;
        for (int i = 0; i < kTableSize; i++) sorted_list_size += table_counter[i] + 1;
        std::vector<watershed_edge> sorted_list(sorted_list_size + 1);
        int max_watershed = -1;
        Data d;
        d.outlog = fopen("/dev/null", "w");
        d.sinkcount = 0;
        sorted_list_size = init_and_sort_watershed_bound_labelsMFD(&d, hash.data(), table_counter.data(), kTableSize,
                                                                   kListSize, sorted_list.data(), sorted_list_size,
                                                                   &max_watershed, counter);
        fclose(d.outlog);
        s->sinkcount = d.sinkcount;
        union_set set(max_watershed + 1);
        std::vector<int> done(max_watershed + 1, 0);
        std::vector<double> raise(std::max((size_t)max_watershed + 1, g.N + 2), 0.0);
        done[0] = 1;
        for (int i = 0; i < sorted_list_size; i++) {  // routeflow.cu:531-566
            int label1 = sorted_list[i].get_node1(), label2 = sorted_list[i].get_node2();
            double height = sorted_list[i].get_weight();
            if (!(set.in_set(label1))) set.make_set(label1);
            if (!(set.in_set(label2))) set.make_set(label2);
            int root1 = set.find_root(label1), root2 = set.find_root(label2);
            if (done[root1] && done[root2]) continue;
            if (done[root1] || done[root2]) {
                if (done[root1]) {
                    done[root2] = 1;
                    raise[root2] = height;
                } else {
                    done[root1] = 1;
                    raise[root1] = height;
                }
                continue;
            }
            if (root1 != root2) {
                set.merge(root1, root2);
                raise[root2] = raise[root1] = height;
            }
        }
        for (int i = 0; i < max_watershed + 1; i++)
            if (raise[i] != 0) raise[i] = raise[set.find_root(i)];
        ref_launch(g.grid, g.block, raise_watershedMFD, mask.data(), ws.data(), raise.data(), dem.data(), g.W, g.H);
        int s2 = 0, f2 = 0;
        ref_launch(g.grid, g.block, FlowDirs, mask.data(), flatmask.data(), dem.data(), slopes.data(), sfd.data(),
                   fd.data(), 1, csize, g.W, g.H, kXmove, kYmove, 0, &s2, &f2);
        plateau_loop(g, mask, dem, slopes, fd, sfd, sp, low, csize, &sweeps);
        if (s->watershed) std::copy(ws.begin(), ws.begin() + g.N, s->watershed);
    }
    s->plateau_sweeps = sweeps;
    if (s->dem_routed) std::copy(dem.begin(), dem.begin() + g.N, s->dem_routed);
    if (s->shortest_paths)
        for (size_t i = 0; i < g.N; ++i) s->shortest_paths[i] = mask[i] == 1 ? sp[i] : 0.f;
    for (size_t i = 0; i < g.N; ++i) {  // routeflow.cu:934-953
        s->sfd[i] = sfd[i];
        s->fd[i] = fd[i];
    }
    if (p->flow_direction_type == 0) {
        for (size_t i = 0; i < g.N; ++i) s->fd[i] = s->sfd[i];
    } else {
        for (size_t i = 0; i < g.N; ++i)
            if (s->fd[i] <= 0 && s->mask[i] == 1) s->fd[i] = s->sfd[i];
    }
    s->fd[s->outlet] = 16;
    return 0;
}

int ref_flow_accumulation(oracle_state* s, const lem_params* p, uint32_t flags) {
    const G g = geom(s);
    std::vector<int> mask = pad_copy(s->mask, g.N, g.pad, 0);
    std::vector<double> rain = pad_copy(s->rainmat, g.N, g.pad, -9999.0);
    std::vector<double> stone = pad_copy(s->stone, g.N, g.pad, 0.0);
    std::vector<double> totB = pad_copy(s->totB, g.N, g.pad, 0.0);
    std::vector<double> soilM = pad_copy(s->soilM, g.N, g.pad, 0.0);
    std::vector<double> w(g.N + g.pad, 0.0);
    const double rescale = 1 / (10000 / (s->cellsize * s->cellsize));
    ref_launch(g.grid, g.block, calcrunoffweight, g.W, g.H, rain.data(), mask.data(), stone.data(), totB.data(),
               soilM.data(), w.data(), rescale);
    std::copy(soilM.begin(), soilM.begin() + g.N, s->soilM);
    std::copy(w.begin(), w.begin() + g.N, s->runoff);
    std::vector<int> fd = pad_copy(s->fd, g.N, g.pad, -9999);
    if (p->flow_direction_type != 0 && p->mfd_proportions) {
        DataProps dp{{g.W, g.H}, s->mask, s->slopes, s->prop, s->fd};
        calcprops(&dp);
    } else {
        for (size_t i = 0; i < g.N; i++)  // calcpropsSFD (runoffweight.cu:115-138)
            for (int k = 0; k < 8; k++) s->prop[i * 8 + k] = (s->mask[i] == 1) ? 1 : 0;
    }
    std::vector<double> prop = pad_copy(s->prop, 8 * g.N, 8 * g.pad, 0.0);
    std::vector<double> fa(g.N + g.pad, 0.0);
    std::vector<double> dem = pad_copy(s->dem, g.N, g.pad, -9999.0);
    std::vector<int> okgrid(g.N + g.pad, 1), localOK(g.N + g.pad, 1);
    for (size_t x = 0; x < g.N; ++x) {
        okgrid[x] = localOK[x] = (s->dem[x] == -9999) ? 1 : 0;
    }
    auto process = [&]() {  // processtheGrid (mfd_simple.cu:174-235) with loopMax = 1
        std::vector<int> ok = okgrid, lok = localOK;
        unsigned int progress;
        int grid_progress = 0, oneZero = 0, oneZero2 = 0;
        do {
            progress = 0;
            oneZero2 = oneZero;
            ref_launch(g.grid, g.block, CalcMFD, mask.data(), dem.data(), fd.data(), fa.data(), prop.data(), ok.data(),
                       &progress, lok.data(), g.W, g.H, w.data());
            grid_progress += progress;
            if (progress == 0)
                oneZero = 1;
            else {
                oneZero = 0;
                oneZero2 = 0;
            }
        } while (progress > 5 || !oneZero2);
        okgrid = ok;
        return grid_progress;
    };
    int gp;
    do {
        gp = process();
        if (gp != 0) gp += process();
    } while (gp > 5);
    long active = 0, undone = 0;
    for (size_t i = 0; i < g.N; ++i) {
        active += s->mask[i] != 0;
        if (okgrid[i] != 1 && s->mask[i] != 0) undone++;
    }
    s->fa_uncomputed = (int)undone;
    std::copy(fa.begin(), fa.begin() + g.N, s->fa);
    double m = 0.0;
    int idx = 0;
    for (size_t i = 0; i < g.N; ++i)
        if (s->fa[i] > m) {
            m = s->fa[i];
            idx = (int)i;
        }
    s->FA_max = m;
    if (flags & LEM_STEP_SET_OUTLET_FROM_FA) s->outlet = idx;
    return 0;
}

int ref_erosion(oracle_state* s, lem_params* p) {
    const G g = geom(s);
    const double cs = s->cellsize;
    const size_t N = g.N, P = g.pad;
    for (size_t i = 0; i < N; i++) {  // aveslope (eroincidep.cu:8-37)
        s->slopeptr[i] = 0.0;
        if (s->mask[i] == 1) {
            double total = 0;
            int nonzero = 0;
            for (int j = 0; j < 8; j++) {
                total += s->slopes[i * 8 + j];
                if (s->slopes[i * 8 + j] > 0) nonzero++;
            }
            if ((total > 0) && (nonzero > 0)) s->slopeptr[i] = total / nonzero;
        }
    }
    std::vector<int> mask = pad_copy(s->mask, N, P, 0);
    std::vector<double> fa = pad_copy(s->fa, N, P, 0.0), sp = pad_copy(s->slopeptr, N, P, 0.0);
    std::vector<double> fines = pad_copy(s->fines, N, P, 0.0), nut = pad_copy(s->nut, N, P, 0.0);
    std::vector<double> soilT = pad_copy(s->soilT, N, P, 0.0), stone = pad_copy(s->stone, N, P, 0.0);
    std::vector<double> totB = pad_copy(s->totB, N, P, 0.0), soilM = pad_copy(s->soilM, N, P, 0.0);
    std::vector<double> soilB = pad_copy(s->soilB, N, P, 0.0);
    std::vector<double> temp = pad_copy(s->tempmat, N, P, -9999.0), rain = pad_copy(s->rainmat, N, P, -9999.0);
    std::vector<double> ltemp = pad_copy(s->last_tempmat, N, P, -9999.0);
    std::vector<double> lrain = pad_copy(s->last_rainmat, N, P, -9999.0);
    std::vector<double> ero(N + P, 0.0), inci(N + P, 0.0), geli(N + P, 0.0), dz(N + P, 0.0);
    std::vector<double> wC(N + P, 0.0), wP(N + P, 0.0);
    std::vector<double> depo = pad_copy(s->depo, N, P, 0.0);
    std::vector<double> dem = pad_copy(s->dem, N, P, -9999.0);
    std::vector<int> fd = pad_copy(s->fd, N, P, -9999);
    std::vector<double> prop = pad_copy(s->prop, 8 * N, 8 * P, 0.0);
    ref_launch(g.grid, g.block, diff_erosion, mask.data(), ero.data(), fa.data(), sp.data(), fines.data(), nut.data(),
               soilT.data(), stone.data(), totB.data(), p->soil_struct, p->profile_permeability, g.W, g.H,
               p->q_threshold);
    ref_launch(g.grid, g.block, conc_erosion, mask.data(), inci.data(), fa.data(), sp.data(), totB.data(),
               soilT.data(), g.W, g.H, cs, p->q_threshold, p->flow_a, p->flow_b, (double*)nullptr, p->max_incision);
    ref_launch(g.grid, g.block, gelifluction, mask.data(), geli.data(), temp.data(), ero.data(), soilT.data(), sp.data(),
               g.W, g.H, fa.data(), s->FA_max, p->g_slope, p->kappa, p->g_flowlim);
    double tE = 0, tI = 0, tG = 0;
    for (size_t i = 0; i < N; ++i) {
        tE += ero[i];
        tI += inci[i];
        tG += geli[i];
    }
    s->totE = tE;
    s->totI = tI;
    s->totG = tG;
    // sedmfdaccum (mfd_accum.cu:345-436)
    std::vector<int> okgrid(N + P, 0), localOK(N + P, 0);
    for (size_t x = 0; x < N; ++x)
        if (s->mask[x] == 1) depo[x] = 0.00001;
    if (p->ddk > 0.95) p->ddk = 0.95;
    if (p->dck > 0.9) p->dck = 0.9;
    auto process = [&]() {
        std::vector<int> ok = okgrid, lok = localOK;
        unsigned int progress;
        int grid_progress = 0, oneZero = 0, oneZero2 = 0;
        do {
            progress = 0;
            oneZero2 = oneZero;
            ref_launch(g.grid, g.block, MFDsedbud, mask.data(), dem.data(), fd.data(), prop.data(), ero.data(),
                       inci.data(), geli.data(), depo.data(), ok.data(), &progress, lok.data(), p->ddk, p->dck,
                       p->dgk, fines.data(), stone.data(), nut.data(), soilT.data(), g.W, g.H);
            grid_progress += progress;
            if (progress == 0)
                oneZero = 1;
            else {
                oneZero = 0;
                oneZero2 = 0;
            }
        } while (progress > 10 || !oneZero2);
        okgrid = ok;
        return grid_progress;
    };
    int gp;
    do {
        gp = process();
        if (gp != 0) gp += process();
    } while (gp > 0);
    long undone = 0;
    for (size_t i = 0; i < N; ++i)
        if (okgrid[i] != 1 && s->mask[i] != 0) undone++;
    s->sed_uncomputed = (int)undone;
    double tD = 0;
    for (size_t i = 0; i < N; ++i) tD += depo[i];
    s->totD = tD;
    ref_launch(g.grid, g.block, surface_change, mask.data(), dz.data(), ero.data(), inci.data(), depo.data(),
               geli.data(), g.H, g.W);
    const double rescale_w = 10000 * (10000 / (cs * cs));
    ref_launch(g.grid, g.block, weathering, mask.data(), temp.data(), rain.data(), fa.data(), 1, wC.data(), wP.data(),
               soilT.data(), fines.data(), stone.data(), soilM.data(), ero.data(), dz.data(), cs, g.H, g.W, rescale_w);
    double tWC = 0, tWP = 0;
    for (size_t i = 0; i < N; ++i) {
        tWC += wC[i];
        tWP += wP[i];
    }
    s->totWC = tWC;
    s->totWP = tWP;
    const double base_level = s->dem[s->outlet] - 0.00012;  // updates.cu:151-174
    ref_launch(g.grid, g.block, Update_Surface, mask.data(), base_level, wC.data(), wP.data(), dem.data(), dz.data(), cs,
               g.H, g.W);
    std::copy(dem.begin(), dem.begin() + N, s->dem);
    s->dem[s->outlet] = base_level;
    s->dem[s->outlet] = s->dem[s->outlet] - 0.00012;
    ref_launch(g.grid, g.block, update_nutrient_content, mask.data(), temp.data(), nut.data(), soilT.data(),
               soilB.data(), totB.data(), g.H, g.W);
    ref_launch(g.grid, g.block, grow_vegetation, mask.data(), temp.data(), ltemp.data(), rain.data(), lrain.data(),
               totB.data(), g.H, g.W, p->temp_inflex, p->temp_sens, (10000 / (cs * cs)));
    double tB = 0;
    for (size_t i = 0; i < N; ++i) tB += totB[i];
    s->totbio = tB;
    auto out = [&](std::vector<double>& v, double* d) { std::copy(v.begin(), v.begin() + N, d); };
    out(ero, s->ero);
    out(inci, s->inci);
    out(geli, s->geli);
    out(depo, s->depo);
    out(dz, s->dz);
    out(wC, s->wC);
    out(wP, s->wP);
    out(soilT, s->soilT);
    out(stone, s->stone);
    out(fines, s->fines);
    out(soilM, s->soilM);
    out(soilB, s->soilB);
    out(nut, s->nut);
    out(totB, s->totB);
    return 0;
}

}  // extern "C"
