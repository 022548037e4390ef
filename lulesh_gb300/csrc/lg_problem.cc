// lg_problem.cc -- host-side Sedov problem set-up and the end-of-run report.
#include "lg_problem.h"

#include <algorithm>
#include <map>

#include <cmath>
#include <cstdio>
#include <sstream>
#include <iomanip>

namespace lg {

// glibc random_r TYPE_3 (degree 31, separation 3): the state is seeded by the
// Park-Miller minimal-standard LCG (16807 mod 2^31-1, Schrage's method), seed
// 0 is treated as 1, the first 310 outputs are discarded, and each output is
// (r[i-31] + r[i-3]) mod 2^32 shifted right by one bit.
GlibcRand::GlibcRand(unsigned seed)
{
    int32_t s = static_cast<int32_t>(seed == 0 ? 1 : seed);
    int32_t st[34];
    st[0] = s;
    for (int i = 1; i < 31; ++i) {
        const int32_t hi = st[i - 1] / 127773;
        const int32_t lo = st[i - 1] % 127773;
        int32_t w = 16807 * lo - 2836 * hi;
        if (w < 0) w += 2147483647;
        st[i] = w;
    }
    // ring of the last 34 words; positions 31..33 repeat 0..2
    for (int i = 31; i < 34; ++i) st[i] = st[i - 31];
    for (int i = 0; i < 34; ++i) r_[i] = st[i];
    i_ = 34;
    for (int k = 0; k < 310; ++k) next();
}

int GlibcRand::next()
{
    // r[i] = r[i-31] + r[i-3]; ring index modulo 34
    const uint32_t a = static_cast<uint32_t>(r_[(i_ - 31) % 34]);
    const uint32_t b = static_cast<uint32_t>(r_[(i_ - 3) % 34]);
    const uint32_t v = a + b;
    r_[i_ % 34] = static_cast<int32_t>(v);
    ++i_;
    if (i_ >= 34 * 1000000) i_ = 34 + (i_ % 34);
    return static_cast<int>(v >> 1);
}

double elem_volume_host(const double x[8], const double y[8], const double z[8])
{
    const double twelveth = 1.0 / 12.0;
    const double dx61 = x[6] - x[1], dy61 = y[6] - y[1], dz61 = z[6] - z[1];
    const double dx70 = x[7] - x[0], dy70 = y[7] - y[0], dz70 = z[7] - z[0];
    const double dx63 = x[6] - x[3], dy63 = y[6] - y[3], dz63 = z[6] - z[3];
    const double dx20 = x[2] - x[0], dy20 = y[2] - y[0], dz20 = z[2] - z[0];
    const double dx50 = x[5] - x[0], dy50 = y[5] - y[0], dz50 = z[5] - z[0];
    const double dx64 = x[6] - x[4], dy64 = y[6] - y[4], dz64 = z[6] - z[4];
    const double dx31 = x[3] - x[1], dy31 = y[3] - y[1], dz31 = z[3] - z[1];
    const double dx72 = x[7] - x[2], dy72 = y[7] - y[2], dz72 = z[7] - z[2];
    const double dx43 = x[4] - x[3], dy43 = y[4] - y[3], dz43 = z[4] - z[3];
    const double dx57 = x[5] - x[7], dy57 = y[5] - y[7], dz57 = z[5] - z[7];
    const double dx14 = x[1] - x[4], dy14 = y[1] - y[4], dz14 = z[1] - z[4];
    const double dx25 = x[2] - x[5], dy25 = y[2] - y[5], dz25 = z[2] - z[5];
    auto tp = [](double a1, double b1, double c1, double a2, double b2, double c2, double a3,
                 double b3, double c3) {
        return a1 * (b2 * c3 - c2 * b3) + a2 * (c1 * b3 - b1 * c3) + a3 * (b1 * c2 - c1 * b2);
    };
    double volume = tp(dx31 + dx72, dx63, dx20, dy31 + dy72, dy63, dy20, dz31 + dz72, dz63, dz20) +
                    tp(dx43 + dx57, dx64, dx70, dy43 + dy57, dy64, dy70, dz43 + dz57, dz64, dz70) +
                    tp(dx14 + dx25, dx61, dx50, dy14 + dy25, dy61, dy50, dz14 + dz25, dz61, dz50);
    volume *= twelveth;
    return volume;
}

int region_rep(int r, int numReg, int cost)
{
    if (r < numReg / 2) return 1;
    if (r < (numReg - (numReg + 15) / 20)) return 1 + cost;
    return 10 * (1 + cost);
}

std::vector<int> region_visit_order(int numReg, int cost)
{
    std::vector<int> order(numReg);
    for (int r = 0; r < numReg; ++r) order[r] = r;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return region_rep(a, numReg, cost) > region_rep(b, numReg, cost);
    });
    return order;
}

bool build_material_items(const Problem &p, long long resident, std::vector<int> &item_elem,
                          std::vector<int> &item_rep)
{
    // elements per repetition count
    std::map<int, long long> count;
    for (int r = 0; r < p.numReg; ++r)
        count[region_rep(r, p.numReg, p.cost)] += (long long)p.regElemlist[r].size();
    const long long T = 3 * resident / 8;
    bool split = false;
    for (const auto &kv : count)
        if (kv.first >= 2 && kv.second > 0 && kv.second < T) split = true;
    item_elem.clear();
    item_rep.clear();
    if (!split) {
        // one item per element, in region visit order (each region's
        // elements in their ascending regElemlist order)
        item_elem.reserve(p.numElem);
        item_rep.reserve(p.numElem);
        for (const int r : region_visit_order(p.numReg, p.cost)) {
            const int rr = region_rep(r, p.numReg, p.cost);
            for (int e : p.regElemlist[r]) {
                item_elem.push_back(e);
                item_rep.push_back(rr);
            }
        }
        return false;
    }
    // repetition items of at most R repetitions: the element's repetitions
    // in near-equal shares, its first item the writer; R keeps the count
    // near 4 x resident or below
    long long total = 0;
    for (const auto &kv : count) total += (long long)kv.first * kv.second;
    const long long R = std::max<long long>(1, (total + 4 * resident - 1) / (4 * resident));
    std::vector<int> region_of(p.numElem, 0);
    for (int r = 0; r < p.numReg; ++r)
        for (int e : p.regElemlist[r]) region_of[e] = r;
    struct Item {
        int elem, share;
        bool writer;
    };
    std::vector<Item> items;
    for (int e = 0; e < p.numElem; ++e) {
        const int rr = region_rep(region_of[e], p.numReg, p.cost);
        const int n = (int)((rr + R - 1) / R);
        for (int i = 0; i < n; ++i)
            items.push_back({e, rr / n + (i < rr % n ? 1 : 0), i == 0});
    }
    // the largest shares first, so that a warp's items carry equal shares
    std::stable_sort(items.begin(), items.end(),
                     [](const Item &a, const Item &b) { return a.share > b.share; });
    item_elem.reserve(items.size());
    item_rep.reserve(items.size());
    for (const Item &it : items) {
        item_elem.push_back(it.elem);
        item_rep.push_back(it.writer ? it.share : -it.share);
    }
    return true;
}

void build_corner_list(Problem &p)
{
    const int N = p.numNode, E = p.numElem;
    std::vector<int> count(N, 0);
    for (int i = 0; i < 8 * E; ++i) ++count[p.nodelist[i]];
    p.nodeElemStart.assign(N + 1, 0);
    for (int i = 1; i <= N; ++i) p.nodeElemStart[i] = p.nodeElemStart[i - 1] + count[i - 1];
    p.nodeElemCornerList.assign(p.nodeElemStart[N], 0);
    std::fill(count.begin(), count.end(), 0);
    for (int i = 0; i < E; ++i)
        for (int j = 0; j < 8; ++j) {
            const int m = p.nodelist[8 * i + j];
            p.nodeElemCornerList[p.nodeElemStart[m] + count[m]++] = 8 * i + j;
        }
}

void build_region_sets(Problem &p)
{
    p.regElemSize.assign(p.numReg, 0);
    for (int i = 0; i < p.numElem; ++i) p.regElemSize[p.regNumList[i] - 1]++;
    p.regElemlist.assign(p.numReg, std::vector<int>());
    for (int r = 0; r < p.numReg; ++r) p.regElemlist[r].reserve(p.regElemSize[r]);
    for (int i = 0; i < p.numElem; ++i) p.regElemlist[p.regNumList[i] - 1].push_back(i);
}

// CreateRegionIndexSets, lulesh-init.cc:401-490 (rank 0, no rotation)
static void draw_regions(Problem &p, int nr, int balance)
{
    GlibcRand rng(0);
    p.numReg = nr;
    p.regNumList.assign(p.numElem, 0);
    int nextIndex = 0;
    if (nr == 1) {
        while (nextIndex < p.numElem) p.regNumList[nextIndex++] = 1;
    } else {
        int lastReg = -1;
        int costDenominator = 0;
        std::vector<int> regBinEnd(nr);
        for (int i = 0; i < nr; ++i) {
            costDenominator += std::pow((i + 1), balance);
            regBinEnd[i] = costDenominator;
        }
        auto pick = [&]() {
            const int regionVar = rng.next() % costDenominator;
            int i = 0;
            while (regionVar >= regBinEnd[i]) i++;
            return (i % nr) + 1;
        };
        while (nextIndex < p.numElem) {
            int regionNum = pick();
            while (regionNum == lastReg) regionNum = pick();
            const int binSize = rng.next() % 1000;
            int elements;
            if (binSize < 773)
                elements = rng.next() % 15 + 1;
            else if (binSize < 937)
                elements = rng.next() % 16 + 16;
            else if (binSize < 970)
                elements = rng.next() % 32 + 32;
            else if (binSize < 974)
                elements = rng.next() % 64 + 64;
            else if (binSize < 978)
                elements = rng.next() % 128 + 128;
            else if (binSize < 981)
                elements = rng.next() % 256 + 256;
            else
                elements = rng.next() % 1537 + 512;
            const int runto = elements + nextIndex;
            while (nextIndex < runto && nextIndex < p.numElem) p.regNumList[nextIndex++] = regionNum;
            lastReg = regionNum;
        }
    }
    build_region_sets(p);
}

Problem build_sedov(int nx, int numReg, int balance, int cost, double hgcoef,
                    double einit_factor)
{
    Problem p;
    const int edgeElems = nx, edgeNodes = nx + 1;
    p.nx = nx;
    p.balance = balance;
    p.cost = cost;
    p.k.hgcoef = hgcoef;
    p.numElem = edgeElems * edgeElems * edgeElems;
    p.numNode = edgeNodes * edgeNodes * edgeNodes;
    const int E = p.numElem, N = p.numNode;

    for (auto *f : {&p.x, &p.y, &p.z, &p.xd, &p.yd, &p.zd, &p.xdd, &p.ydd, &p.zdd, &p.fx, &p.fy,
                    &p.fz, &p.nodalMass})
        f->assign(N, 0.0);
    for (auto *f : {&p.e, &p.p, &p.q, &p.ql, &p.qq, &p.v, &p.volo, &p.vnew, &p.delv, &p.vdov,
                    &p.arealg, &p.ss, &p.elemMass})
        f->assign(E, 0.0);
    std::fill(p.v.begin(), p.v.end(), 1.0);

    // BuildMesh, lulesh-init.cc:218-267
    int nidx = 0;
    double tz = 0.0;
    for (int plane = 0; plane < edgeNodes; ++plane) {
        double ty = 0.0;
        for (int row = 0; row < edgeNodes; ++row) {
            double tx = 0.0;
            for (int col = 0; col < edgeNodes; ++col) {
                p.x[nidx] = tx;
                p.y[nidx] = ty;
                p.z[nidx] = tz;
                ++nidx;
                tx = 1.125 * double(col + 1) / double(nx);
            }
            ty = 1.125 * double(row + 1) / double(nx);
        }
        tz = 1.125 * double(plane + 1) / double(nx);
    }
    p.nodelist.assign(8 * (size_t)E, 0);
    int zidx = 0;
    nidx = 0;
    for (int plane = 0; plane < edgeElems; ++plane) {
        for (int row = 0; row < edgeElems; ++row) {
            for (int col = 0; col < edgeElems; ++col) {
                int *ln = &p.nodelist[8 * (size_t)zidx];
                ln[0] = nidx;
                ln[1] = nidx + 1;
                ln[2] = nidx + edgeNodes + 1;
                ln[3] = nidx + edgeNodes;
                ln[4] = nidx + edgeNodes * edgeNodes;
                ln[5] = nidx + edgeNodes * edgeNodes + 1;
                ln[6] = nidx + edgeNodes * edgeNodes + edgeNodes + 1;
                ln[7] = nidx + edgeNodes * edgeNodes + edgeNodes;
                ++zidx;
                ++nidx;
            }
            ++nidx;
        }
        nidx += edgeNodes;
    }
    build_corner_list(p);
    draw_regions(p, numReg, balance);

    // SetupSymmetryPlanes, lulesh-init.cc:514-533
    const int nsymm = edgeNodes * edgeNodes;
    p.symmX.assign(nsymm, 0);
    p.symmY.assign(nsymm, 0);
    p.symmZ.assign(nsymm, 0);
    nidx = 0;
    for (int i = 0; i < edgeNodes; ++i) {
        const int planeInc = i * edgeNodes * edgeNodes, rowInc = i * edgeNodes;
        for (int j = 0; j < edgeNodes; ++j) {
            p.symmZ[nidx] = rowInc + j;
            p.symmY[nidx] = planeInc + j;
            p.symmX[nidx] = planeInc + j * edgeNodes;
            ++nidx;
        }
    }

    // SetupElementConnectivities, lulesh-init.cc:539-565
    for (auto *f : {&p.lxim, &p.lxip, &p.letam, &p.letap, &p.lzetam, &p.lzetap}) f->assign(E, 0);
    const int n = edgeElems;
    p.lxim[0] = 0;
    for (int i = 1; i < E; ++i) {
        p.lxim[i] = i - 1;
        p.lxip[i - 1] = i;
    }
    p.lxip[E - 1] = E - 1;
    for (int i = 0; i < n; ++i) {
        p.letam[i] = i;
        p.letap[E - n + i] = E - n + i;
    }
    for (int i = n; i < E; ++i) {
        p.letam[i] = i - n;
        p.letap[i - n] = i;
    }
    for (int i = 0; i < n * n; ++i) {
        p.lzetam[i] = i;
        p.lzetap[E - n * n + i] = E - n * n + i;
    }
    for (int i = n * n; i < E; ++i) {
        p.lzetam[i] = i - n * n;
        p.lzetap[i - n * n] = i;
    }

    // SetupBoundaryConditions, lulesh-init.cc:569-673 (min faces symmetric,
    // max faces free on a single rank)
    p.elemBC.assign(E, 0);
    for (int i = 0; i < n; ++i) {
        const int planeInc = i * n * n, rowInc = i * n;
        for (int j = 0; j < n; ++j) {
            p.elemBC[rowInc + j] |= ZETA_M_SYMM;
            p.elemBC[rowInc + j + E - n * n] |= ZETA_P_FREE;
            p.elemBC[planeInc + j] |= ETA_M_SYMM;
            p.elemBC[planeInc + j + n * n - n] |= ETA_P_FREE;
            p.elemBC[planeInc + j * n] |= XI_M_SYMM;
            p.elemBC[planeInc + j * n + n - 1] |= XI_P_FREE;
        }
    }

    // volumes and masses, lulesh-init.cc:159-178 (serial accumulation order)
    for (int i = 0; i < E; ++i) {
        double xl[8], yl[8], zl[8];
        const int *en = &p.nodelist[8 * (size_t)i];
        for (int l = 0; l < 8; ++l) {
            xl[l] = p.x[en[l]];
            yl[l] = p.y[en[l]];
            zl[l] = p.z[en[l]];
        }
        const double volume = elem_volume_host(xl, yl, zl);
        p.volo[i] = volume;
        p.elemMass[i] = volume;
        for (int j = 0; j < 8; ++j) p.nodalMass[en[j]] += volume / 8.0;
    }

    // deposited energy and analytic first step, lulesh-init.cc:183-192
    const double einit = sedov_einit(nx, einit_factor);
    p.e[0] = einit;
    p.t.deltatime = (.5 * std::cbrt(p.volo[0])) / std::sqrt(2.0 * einit);
    return p;
}

double sedov_einit(int nx, double einit_factor)
{
    const double ebase = 3.948746e+7;
    const double scale = (nx * 1) / 45.0;
    double einit = ebase * scale * scale * scale;
    return einit * einit_factor;
}

Problem build_sedov_scalars(int nx, int numReg, int balance, int cost, double hgcoef,
                            double einit_factor)
{
    Problem p;
    p.nx = nx;
    p.balance = balance;
    p.cost = cost;
    p.k.hgcoef = hgcoef;
    p.numElem = nx * nx * nx;
    p.numNode = (nx + 1) * (nx + 1) * (nx + 1);
    draw_regions(p, numReg, balance);
    // element 0's corners at the BuildMesh coordinates 0 and 1.125 / nx
    const double h = 1.125 * double(1) / double(nx);
    const double x0[8] = {0.0, h, h, 0.0, 0.0, h, h, 0.0};
    const double y0[8] = {0.0, 0.0, h, h, 0.0, 0.0, h, h};
    const double z0[8] = {0.0, 0.0, 0.0, 0.0, h, h, h, h};
    const double volo0 = elem_volume_host(x0, y0, z0);
    const double einit = sedov_einit(nx, einit_factor);
    p.t.deltatime = (.5 * std::cbrt(volo0)) / std::sqrt(2.0 * einit);
    return p;
}

std::string format_report(int nx, int cycle, double e0, double maxAbsDiff, double totalAbsDiff,
                          double maxRelDiff, double elapsed)
{
    // Formatting follows lulesh-util.cc:184-227 (same stream manipulators).
    const long long nx8 = nx;
    const double grindTime1 = ((elapsed * 1e6) / cycle) / double(nx8 * nx8 * nx8);
    const double grindTime2 = ((elapsed * 1e6) / cycle) / double(nx8 * nx8 * nx8 * 1);
    std::ostringstream os;
    os << "Run completed:\n";
    os << "   Problem size        =  " << nx << "\n";
    os << "   MPI tasks           =  " << 1 << "\n";
    os << "   Iteration count     =  " << cycle << "\n";
    os << "   Final Origin Energy =  ";
    os << std::scientific << std::setprecision(6);
    os << std::setw(12) << e0 << "\n";
    os << "   Testing Plane 0 of Energy Array on rank 0:\n";
    os << "        MaxAbsDiff   = " << std::setw(12) << maxAbsDiff << "\n";
    os << "        TotalAbsDiff = " << std::setw(12) << totalAbsDiff << "\n";
    os << "        MaxRelDiff   = " << std::setw(12) << maxRelDiff << "\n";
    os.unsetf(std::ios_base::floatfield);
    os << std::setprecision(2);
    os << "\nElapsed time         = " << std::setw(10) << elapsed << " (s)\n";
    os << std::setprecision(8);
    os << "Grind time (us/z/c)  = " << std::setw(10) << grindTime1 << " (per dom)  ("
       << std::setw(10) << elapsed << " overall)\n";
    os << "FOM                  = " << std::setw(10) << 1000.0 / grindTime2 << " (z/s)\n\n";
    return os.str();
}

}  // namespace lg
