// Host-side geometry plan of the M-Mbulge scatter stage (holodeck/sams/sam.py:1291-1394).
//
// Everything here depends only on the (mtot, mrat) grid edges, the refinement and the scatter
// width, never on the density values, so a plan is built once per grid and reused for every
// redshift slice and every model on that grid:
//   * the points (log10 m1, log10 m2) of the (mtot, mrat) grid and their Delaunay triangulation
//     (incremental Bowyer-Watson insertion in grid order with ghost triangles for the hull, and
//     orientation / in-circle predicates filtered in double precision and re-evaluated in long
//     double when the double result is inside its error bound);
//   * the triangle neighbours, turned into the cross-derivative coefficient of each triangle edge
//     used by the Clough-Tocher evaluation (derivative linear along the edge in the direction of
//     the line joining the centroids of the two triangles sharing it, or of the centroid-to-midpoint
//     direction on hull edges);
//   * per point: the edges to its neighbours (vectors and vector / length^3) and the inverse of the
//     2x2 normal matrix of the minimum-norm-network gradient update (Nielson 1983), and the
//     Gauss-Seidel wavefront levels: level(i) = 1 + max level of the lower-indexed neighbours, so
//     one level's points update concurrently while reading exactly the values a sequential sweep in
//     point order would read;
//   * per node of the regular (log m1, log m2) grid: containing triangle and barycentric
//     coordinates (or -1 outside the hull) and the nearest point (greedy descent on the Delaunay
//     graph, exact for any query point);
//   * per point: the lower grid cell and fractional offsets of the bilinear interpolation back;
//   * the Gaussian redistribution matrix W[i][k] = P(bin k | source bin i) of utils.py:382-488, and
//     per point the row of (W W) that, combined with the bilinear weights, maps a slice's regular
//     grid straight to the point's redistributed value.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "holodeck_gb300.h"

namespace {

struct P2 {
    double x, y;
};

// ---- predicates: double with an error bound, long double when the sign is uncertain
int orient_sign(const P2 &a, const P2 &b, const P2 &c) {
    double dl = (a.x - c.x) * (b.y - c.y);
    double dr = (a.y - c.y) * (b.x - c.x);
    double det = dl - dr;
    double bound = 3.3306690738754716e-16 * (fabs(dl) + fabs(dr));
    if (det > bound) return 1;
    if (-det > bound) return -1;
    long double L = ((long double)a.x - c.x) * ((long double)b.y - c.y) - ((long double)a.y - c.y) * ((long double)b.x - c.x);
    return (L > 0) - (L < 0);
}

int incircle_sign(const P2 &a, const P2 &b, const P2 &c, const P2 &d) {
    double adx = a.x - d.x, ady = a.y - d.y, bdx = b.x - d.x, bdy = b.y - d.y, cdx = c.x - d.x, cdy = c.y - d.y;
    double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy, alift = adx * adx + ady * ady;
    double cdxady = cdx * ady, adxcdy = adx * cdy, blift = bdx * bdx + bdy * bdy;
    double adxbdy = adx * bdy, bdxady = bdx * ady, clift = cdx * cdx + cdy * cdy;
    double det = alift * (bdxcdy - cdxbdy) + blift * (cdxady - adxcdy) + clift * (adxbdy - bdxady);
    double perm = (fabs(bdxcdy) + fabs(cdxbdy)) * alift + (fabs(cdxady) + fabs(adxcdy)) * blift +
                  (fabs(adxbdy) + fabs(bdxady)) * clift;
    double bound = 1.1102230246251577e-15 * perm;
    if (det > bound) return 1;
    if (-det > bound) return -1;
    long double Adx = (long double)a.x - d.x, Ady = (long double)a.y - d.y;
    long double Bdx = (long double)b.x - d.x, Bdy = (long double)b.y - d.y;
    long double Cdx = (long double)c.x - d.x, Cdy = (long double)c.y - d.y;
    long double L = (Adx * Adx + Ady * Ady) * (Bdx * Cdy - Cdx * Bdy) + (Bdx * Bdx + Bdy * Bdy) * (Cdx * Ady - Adx * Cdy) +
                    (Cdx * Cdx + Cdy * Cdy) * (Adx * Bdy - Bdx * Ady);
    return (L > 0) - (L < 0);
}

constexpr int INF = -1;

struct Tri {
    int v[3];   // counter-clockwise; a ghost triangle holds INF as v[2] and its real edge v[0] -> v[1]
    int n[3];   // n[k]: triangle across the edge opposite v[k]
    bool alive;
};

class Triangulation {
   public:
    std::vector<P2> p;
    std::vector<Tri> t;
    std::vector<int> free_slots;
    std::vector<int> mark;   // cavity membership stamps
    std::vector<int> by_a;   // new-triangle lookup by first vertex during one insertion
    int stamp = 0;
    int last = 0;

    int new_tri(int a, int b, int c) {
        Tri tr;
        tr.v[0] = a;
        tr.v[1] = b;
        tr.v[2] = c;
        tr.n[0] = tr.n[1] = tr.n[2] = -1;
        tr.alive = true;
        if (!free_slots.empty()) {
            int id = free_slots.back();
            free_slots.pop_back();
            t[id] = tr;
            return id;
        }
        t.push_back(tr);
        return (int)t.size() - 1;
    }

    static bool is_ghost(const Tri &tr) { return tr.v[0] == INF || tr.v[1] == INF || tr.v[2] == INF; }

    // In conflict = the new point lies strictly inside the triangle's circumcircle (for a ghost:
    // strictly outside its hull edge, or on the open hull edge).
    bool conflict(int id, int ip) const {
        const Tri &tr = t[id];
        const P2 &q = p[ip];
        if (!is_ghost(tr)) return incircle_sign(p[tr.v[0]], p[tr.v[1]], p[tr.v[2]], q) > 0;
        int k = tr.v[0] == INF ? 0 : (tr.v[1] == INF ? 1 : 2);
        int a = tr.v[(k + 1) % 3], b = tr.v[(k + 2) % 3];   // hull edge a -> b with the outside on its left
        int o = orient_sign(p[a], p[b], q);
        if (o > 0) return true;
        if (o < 0) return false;
        // collinear: conflict when q lies strictly inside the segment
        double dx = p[b].x - p[a].x, dy = p[b].y - p[a].y;
        double s = (q.x - p[a].x) * dx + (q.y - p[a].y) * dy;
        return s > 0.0 && s < dx * dx + dy * dy;
    }

    // A triangle in conflict with point ip, found by walking from the last created triangle.
    int locate(int ip) {
        int cur = last;
        if (!t[cur].alive) {
            for (cur = 0; cur < (int)t.size() && !t[cur].alive; cur++) {
            }
        }
        const P2 &q = p[ip];
        for (long guard = 0; guard < 4L * (long)t.size() + 16; guard++) {
            const Tri &tr = t[cur];
            if (is_ghost(tr)) {
                if (conflict(cur, ip)) return cur;
                // step back into the real triangle across the hull edge
                int k = tr.v[0] == INF ? 0 : (tr.v[1] == INF ? 1 : 2);
                cur = tr.n[k];
                continue;
            }
            int next = -1;
            for (int k = 0; k < 3; k++) {
                if (orient_sign(p[tr.v[(k + 1) % 3]], p[tr.v[(k + 2) % 3]], q) < 0) {
                    next = tr.n[k];
                    break;
                }
            }
            if (next < 0) return cur;
            cur = next;
        }
        for (int id = 0; id < (int)t.size(); id++)   // fallback: exhaustive search
            if (t[id].alive && conflict(id, ip)) return id;
        return -1;
    }

    bool init(int i0, int i1, int i2) {
        int o = orient_sign(p[i0], p[i1], p[i2]);
        if (o == 0) return false;
        if (o < 0) std::swap(i1, i2);
        int tr = new_tri(i0, i1, i2);
        int g0 = new_tri(i1, i0, INF);   // across edge i0 -> i1
        int g1 = new_tri(i2, i1, INF);
        int g2 = new_tri(i0, i2, INF);
        // real triangle: n[0] across (i1, i2), n[1] across (i2, i0), n[2] across (i0, i1)
        t[tr].n[0] = g1;
        t[tr].n[1] = g2;
        t[tr].n[2] = g0;
        // ghost (a, b, INF): n[2] across (a, b) = real; n[0] across (b, INF); n[1] across (INF, a)
        t[g0].n[2] = tr;
        t[g1].n[2] = tr;
        t[g2].n[2] = tr;
        t[g0].n[0] = g2;   // g0 = (i1, i0, INF): edge (i0, INF) shared with g2 = (i0, i2, INF) edge (INF, i0)
        t[g2].n[1] = g0;
        t[g0].n[1] = g1;   // edge (INF, i1) shared with g1 = (i2, i1, INF) edge (i1, INF)
        t[g1].n[0] = g0;
        t[g1].n[1] = g2;   // edge (INF, i2) shared with g2 edge (i2, INF)
        t[g2].n[0] = g1;
        last = tr;
        return true;
    }

    bool insert(int ip) {
        int start = locate(ip);
        if (start < 0) return false;
        if (mark.size() < t.size() + 8) mark.resize(2 * t.size() + 64, 0);
        stamp++;
        auto in_cav = [&](int id) { return mark[id] == stamp; };
        std::vector<int> cavity{start}, stack{start};
        mark[start] = stamp;
        while (!stack.empty()) {
            int id = stack.back();
            stack.pop_back();
            for (int k = 0; k < 3; k++) {
                int nb = t[id].n[k];
                if (nb < 0 || in_cav(nb)) continue;
                if (conflict(nb, ip)) {
                    mark[nb] = stamp;
                    cavity.push_back(nb);
                    stack.push_back(nb);
                }
            }
        }
        // boundary edges (a, b) of the cavity, oriented as in the cavity triangle, with the outside neighbour
        struct Edge {
            int a, b, outside;
        };
        std::vector<Edge> edges;
        for (int id : cavity) {
            for (int k = 0; k < 3; k++) {
                int nb = t[id].n[k];
                if (nb >= 0 && in_cav(nb)) continue;
                edges.push_back({t[id].v[(k + 1) % 3], t[id].v[(k + 2) % 3], nb});
            }
        }
        for (int id : cavity) {
            t[id].alive = false;
            free_slots.push_back(id);
        }
        // new triangles (a, b, ip); link to the outside and to each other through shared vertices
        std::vector<int> made(edges.size());
        for (size_t e = 0; e < edges.size(); e++) {
            int id = new_tri(edges[e].a, edges[e].b, ip);
            made[e] = id;
            t[id].n[2] = edges[e].outside;
            if (edges[e].outside >= 0) {
                Tri &o = t[edges[e].outside];
                for (int k = 0; k < 3; k++) {
                    int x = o.v[(k + 1) % 3], y = o.v[(k + 2) % 3];
                    if (x == edges[e].b && y == edges[e].a) o.n[k] = id;
                }
            }
        }
        // (a, b, ip): n[0] across (b, ip) pairs with the new triangle whose a equals this b; the cavity
        // boundary is a closed loop, so every vertex starts exactly one boundary edge
        if (by_a.size() < p.size() + 1) by_a.assign(p.size() + 1, -1);
        auto slot = [&](int v) { return v == INF ? (int)p.size() : v; };
        for (size_t e = 0; e < edges.size(); e++) by_a[slot(edges[e].a)] = (int)e;
        for (size_t e = 0; e < edges.size(); e++) {
            int f = by_a[slot(edges[e].b)];
            t[made[e]].n[0] = made[f];
            t[made[f]].n[1] = made[e];
        }
        for (size_t e = 0; e < edges.size(); e++) by_a[slot(edges[e].a)] = -1;
        for (int id : made)
            if (!is_ghost(t[id])) last = id;
        return true;
    }
};

// first index i with a[i] >= x (numpy.searchsorted, side='left')
int search_left(const std::vector<double> &a, double x) {
    return (int)(std::lower_bound(a.begin(), a.end(), x) - a.begin());
}

// standard normal CDF with the branch structure of the Cephes ndtr routine
double ndtr(double a) {
    double x = a * M_SQRT1_2;
    double z = fabs(x);
    if (z < M_SQRT1_2) return 0.5 + 0.5 * erf(x);
    double y = 0.5 * erfc(z);
    return (x > 0) ? 1.0 - y : y;
}

}  // namespace

extern "C" {

int hgb_scatter_plan_bounds(int n_mtot, int n_mrat, int refine, hgb_scatter_sizes *out) {
    if (!out || n_mtot < 2 || n_mrat < 2 || refine < 1) return HGB_ERR_INVALID_ARGUMENT;
    int n = n_mtot * n_mrat;
    out->n_pts = n;
    out->n_tri = 2 * n;
    out->n_nbr = 6 * n;
    out->n_grid = refine * n_mtot;
    out->n_levels = n;
    return HGB_OK;
}

int hgb_scatter_plan_build(const double *mtot, int n_mtot, const double *mrat, int n_mrat, int refine,
                           double scatter_dex, hgb_scatter_host_plan *plan, hgb_scatter_sizes *sizes) {
    if (!mtot || !mrat || !plan || !sizes || n_mtot < 2 || n_mrat < 2 || refine < 1 || !(scatter_dex > 0.0))
        return HGB_ERR_INVALID_ARGUMENT;
    const int n = n_mtot * n_mrat;
    const int N = refine * n_mtot;

    // ---- points (sam.py:1347-1360): log10 of the component masses, m-major
    Triangulation T;
    T.p.resize(n);
    for (int i = 0; i < n_mtot; i++)
        for (int j = 0; j < n_mrat; j++) {
            double m1 = mtot[i] / (1.0 + mrat[j]);
            double m2 = mtot[i] - m1;
            T.p[i * n_mrat + j] = {log10(m1), log10(m2)};
        }
    std::vector<P2> orig = T.p;
    // shift both axes by one scalar so that points with equal coordinates stay exactly equal
    double shift = 0.0;
    for (auto &q : T.p) shift += q.x;
    shift /= n;
    for (auto &q : T.p) {
        q.x -= shift;
        q.y -= shift;
    }

    // ---- Delaunay triangulation
    int i0 = 0, i1 = 1, i2 = -1;
    for (int k = 2; k < n && i2 < 0; k++)
        if (orient_sign(T.p[i0], T.p[i1], T.p[k]) != 0) i2 = k;
    if (i2 < 0 || !T.init(i0, i1, i2)) return HGB_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < n; k++) {
        if (k == i0 || k == i1 || k == i2) continue;
        if (!T.insert(k)) return HGB_ERR_INVALID_ARGUMENT;
    }
    // Peel near-degenerate slivers off the hull.  Points on the q = min(mrat) edge are collinear
    // up to rounding, and the exact triangulation of their zig-zag has zero-area hull triangles
    // (area / longest edge^2 ~ 1e-13) that qhull merges away; such a triangle is dropped and its
    // neighbours become hull triangles, repeatedly.
    std::vector<char> outside(T.t.size(), 0);
    for (int id = 0; id < (int)T.t.size(); id++)
        outside[id] = !T.t[id].alive || Triangulation::is_ghost(T.t[id]);
    for (bool changed = true; changed;) {
        changed = false;
        for (int id = 0; id < (int)T.t.size(); id++) {
            if (outside[id]) continue;
            const Tri &tr = T.t[id];
            bool on_hull = false;
            for (int k = 0; k < 3; k++)
                if (tr.n[k] < 0 || outside[tr.n[k]]) on_hull = true;
            if (!on_hull) continue;
            const P2 &a = T.p[tr.v[0]], &b = T.p[tr.v[1]], &c = T.p[tr.v[2]];
            double area2 = fabs((b.x - a.x) * (c.y - a.y) - (c.x - a.x) * (b.y - a.y));
            double l2 = std::max({(b.x - a.x) * (b.x - a.x) + (b.y - a.y) * (b.y - a.y),
                                  (c.x - b.x) * (c.x - b.x) + (c.y - b.y) * (c.y - b.y),
                                  (a.x - c.x) * (a.x - c.x) + (a.y - c.y) * (a.y - c.y)});
            if (area2 < 1e-10 * l2) {
                outside[id] = 1;
                changed = true;
            }
        }
    }
    // collect real triangles and renumber
    std::vector<int> remap(T.t.size(), -1);
    std::vector<int> real;
    for (int id = 0; id < (int)T.t.size(); id++)
        if (!outside[id]) {
            remap[id] = (int)real.size();
            real.push_back(id);
        }
    const int ntri = (int)real.size();
    if (ntri > 2 * n) return HGB_ERR_INVALID_ARGUMENT;
    std::vector<P2> cen(ntri);
    for (int r = 0; r < ntri; r++) {
        const Tri &tr = T.t[real[r]];
        for (int k = 0; k < 3; k++) plan->tri[3 * r + k] = tr.v[k];
        cen[r] = {(orig[tr.v[0]].x + orig[tr.v[1]].x + orig[tr.v[2]].x) / 3.0,
                  (orig[tr.v[0]].y + orig[tr.v[1]].y + orig[tr.v[2]].y) / 3.0};
    }
    // cross-derivative coefficient of each edge k (opposite vertex k, from v[k+1] to v[k+2])
    for (int r = 0; r < ntri; r++) {
        const Tri &tr = T.t[real[r]];
        for (int k = 0; k < 3; k++) {
            const P2 &pi = orig[tr.v[(k + 1) % 3]], &pj = orig[tr.v[(k + 2) % 3]];
            double ex = pj.x - pi.x, ey = pj.y - pi.y, ee = ex * ex + ey * ey;
            double dx = cen[r].x - 0.5 * (pi.x + pj.x), dy = cen[r].y - 0.5 * (pi.y + pj.y);
            double mu = (dx * ex + dy * ey) / ee;
            int nb = tr.n[k];
            double kappa = 0.0;
            if (nb >= 0 && remap[nb] >= 0) {
                const P2 &cn = cen[remap[nb]];
                double wx = cn.x - cen[r].x, wy = cn.y - cen[r].y;
                double nx = -ey, ny = ex;
                kappa = mu - (dx * nx + dy * ny) * (wx * ex + wy * ey) / ((wx * nx + wy * ny) * ee);
            }
            plan->tri_kappa[3 * r + k] = kappa;
        }
    }

    // ---- point neighbourhoods, normal matrices, wavefront levels
    std::vector<std::vector<int>> nb(n);
    for (int r = 0; r < ntri; r++)
        for (int k = 0; k < 3; k++) {
            int a = plan->tri[3 * r + k], b = plan->tri[3 * r + (k + 1) % 3];
            nb[a].push_back(b);
            nb[b].push_back(a);
        }
    int nnz = 0;
    std::vector<int> level(n, 0);
    int nlev = 0;
    for (int i = 0; i < n; i++) {
        std::sort(nb[i].begin(), nb[i].end());
        nb[i].erase(std::unique(nb[i].begin(), nb[i].end()), nb[i].end());
        plan->nbr_ptr[i] = nnz;
        double q00 = 0, q01 = 0, q11 = 0;
        int lv = 0;
        for (int j : nb[i]) {
            double ex = orig[j].x - orig[i].x, ey = orig[j].y - orig[i].y;
            double L = sqrt(ex * ex + ey * ey), L3 = L * L * L;
            plan->nbr_idx[nnz] = j;
            plan->nbr_w[4 * nnz + 0] = ex;
            plan->nbr_w[4 * nnz + 1] = ey;
            plan->nbr_w[4 * nnz + 2] = ex / L3;
            plan->nbr_w[4 * nnz + 3] = ey / L3;
            q00 += 4 * ex * ex / L3;
            q01 += 4 * ex * ey / L3;
            q11 += 4 * ey * ey / L3;
            nnz++;
            if (j < i && level[j] + 1 > lv) lv = level[j] + 1;
        }
        level[i] = lv;
        if (lv + 1 > nlev) nlev = lv + 1;
        double det = q00 * q11 - q01 * q01;
        plan->vtx_qinv[4 * i + 0] = q11 / det;
        plan->vtx_qinv[4 * i + 1] = -q01 / det;
        plan->vtx_qinv[4 * i + 2] = -q01 / det;
        plan->vtx_qinv[4 * i + 3] = q00 / det;
    }
    plan->nbr_ptr[n] = nnz;
    {
        std::vector<int> count(nlev + 1, 0);
        for (int i = 0; i < n; i++) count[level[i] + 1]++;
        for (int l = 0; l < nlev; l++) count[l + 1] += count[l];
        for (int l = 0; l <= nlev; l++) plan->level_ptr[l] = count[l];
        std::vector<int> fill(count.begin(), count.end() - 1);
        for (int i = 0; i < n; i++) plan->level_vtx[fill[level[i]]++] = i;
        // level-order copies: a level's points are contiguous, neighbours keep their order
        std::vector<int> pos_of(n);
        for (int p = 0; p < n; p++) pos_of[plan->level_vtx[p]] = p;
        int e = 0;
        for (int p = 0; p < n; p++) {
            const int i = plan->level_vtx[p];
            plan->lv_nbr_ptr[p] = e;
            for (int q = plan->nbr_ptr[i]; q < plan->nbr_ptr[i + 1]; q++, e++) {
                plan->lv_nbr[e] = pos_of[plan->nbr_idx[q]];
                // -2 w0, -2 w1, w2, w3: the level-order solve folds the factor -2 into its weights
                for (int c = 0; c < 4; c++) plan->lv_nbr_w[4 * e + c] = (c < 2 ? -2.0 : 1.0) * plan->nbr_w[4 * q + c];
            }
            for (int c = 0; c < 4; c++) plan->lv_qinv[4 * p + c] = plan->vtx_qinv[4 * i + c];
        }
        plan->lv_nbr_ptr[n] = e;
    }

    // ---- regular (log m1, log m2) grid (sam.py:1349-1357)
    double lo = 0.9 * mtot[0] * mrat[0] / (1.0 + mrat[0]);
    double hi = mtot[n_mtot - 1] * (1.0 + mrat[0]) / mrat[0];
    if (lo > hi) std::swap(lo, hi);
    double llo = log10(lo), lhi = log10(hi);
    std::vector<double> axis(N);
    double step = (lhi - llo) / (N - 1);
    for (int k = 0; k < N; k++) axis[k] = log10(pow(10.0, (k == N - 1) ? lhi : llo + k * step));
    for (int k = 0; k < N; k++) plan->grid_axis[k] = axis[k];

    // containing triangle + barycentric coordinates of every node (walk through the triangulation)
    {
        int cur = T.last;
        for (int a = 0; a < N; a++) {
            for (int b = 0; b < N; b++) {
                P2 q = {axis[a] - shift, axis[b] - shift};
                int found = -1;
                if (outside[cur]) cur = real[0];
                for (long guard = 0; guard < 4L * ntri + 16; guard++) {
                    const Tri &tr = T.t[cur];
                    int next = -2;
                    for (int k = 0; k < 3; k++) {
                        if (orient_sign(T.p[tr.v[(k + 1) % 3]], T.p[tr.v[(k + 2) % 3]], q) < 0) {
                            next = tr.n[k];
                            break;
                        }
                    }
                    if (next == -2) {
                        found = cur;
                        break;
                    }
                    if (next < 0 || outside[next]) break;   // left the hull
                    cur = next;
                }
                long g = (long)a * N + b;
                if (found < 0) {
                    plan->grid_tri[g] = -1;
                    plan->grid_bary[3 * g + 0] = plan->grid_bary[3 * g + 1] = plan->grid_bary[3 * g + 2] = 0.0;
                    continue;
                }
                int r = remap[found];
                plan->grid_tri[g] = r;
                const P2 &p0 = orig[plan->tri[3 * r]], &p1 = orig[plan->tri[3 * r + 1]], &p2 = orig[plan->tri[3 * r + 2]];
                // c = inv([[x0-x2, x1-x2], [y0-y2, y1-y2]]) (q - p2)
                double a11 = p0.x - p2.x, a12 = p1.x - p2.x, a21 = p0.y - p2.y, a22 = p1.y - p2.y;
                double det = a11 * a22 - a12 * a21;
                double qx = axis[a] - p2.x, qy = axis[b] - p2.y;
                double c0 = (a22 * qx - a12 * qy) / det;
                double c1 = (-a21 * qx + a11 * qy) / det;
                plan->grid_bary[3 * g + 0] = c0;
                plan->grid_bary[3 * g + 1] = c1;
                plan->grid_bary[3 * g + 2] = 1.0 - c0 - c1;
            }
        }
    }

    // nearest point of every node: greedy descent on the Delaunay graph (before the sliver peel),
    // which ends at the exact nearest point of any query; each node starts from its predecessor's
    // answer, so descents are a few steps long
    {
        std::vector<std::vector<int>> adj(n);
        for (int id = 0; id < (int)T.t.size(); id++) {
            const Tri &tr = T.t[id];
            if (!tr.alive || Triangulation::is_ghost(tr)) continue;
            for (int k = 0; k < 3; k++) {
                adj[tr.v[k]].push_back(tr.v[(k + 1) % 3]);
                adj[tr.v[(k + 1) % 3]].push_back(tr.v[k]);
            }
        }
        auto d2 = [&](int i, double x, double y) {
            double dx = orig[i].x - x, dy = orig[i].y - y;
            return dx * dx + dy * dy;
        };
        int cur = 0;
        for (int a = 0; a < N; a++) {
            int row_start = -1;
            for (int b = 0; b < N; b++) {
                double x = axis[a], y = axis[b];
                double bd = d2(cur, x, y);
                for (bool moved = true; moved;) {
                    moved = false;
                    for (int j : adj[cur]) {
                        double dj = d2(j, x, y);
                        if (dj < bd || (dj == bd && j < cur)) {
                            bd = dj;
                            cur = j;
                            moved = true;
                        }
                    }
                }
                plan->grid_near[(long)a * N + b] = cur;
                if (b == 0) row_start = cur;
            }
            cur = row_start;
        }
    }

    // bilinear interpolation back to the points (RegularGridInterpolator, method='linear')
    for (int i = 0; i < n; i++) {
        double xy[2] = {orig[i].x, orig[i].y};
        for (int d = 0; d < 2; d++) {
            int k = search_left(axis, xy[d]) - 1;
            if (k < 0) k = 0;
            if (k > N - 2) k = N - 2;
            plan->back_idx[2 * i + d] = k;
            plan->back_t[2 * i + d] = (xy[d] - axis[k]) / (axis[k + 1] - axis[k]);
        }
    }

    // Gaussian redistribution weights (utils.py:410-488): dm over bin edges at +-(dx/2 + k dx)
    {
        double dx = axis[1] - axis[0];
        std::vector<double> edges(2 * N), cdf(2 * N), dm(2 * N - 1);
        for (int k = 0; k < N; k++) {
            double e = dx / 2.0 + k * dx;
            edges[N + k] = e;
            edges[N - 1 - k] = -e;
        }
        for (int k = 0; k < 2 * N; k++) cdf[k] = ndtr(edges[k] / scatter_dex);
        for (int k = 0; k < 2 * N - 1; k++) dm[k] = cdf[k + 1] - cdf[k];
        for (int i = 0; i < N; i++)
            for (int k = 0; k < N; k++) plan->weights[(long)i * N + k] = dm[k - i + N - 1];
    }

    // The reference redistributes the primary-mass axis twice (see hgb_add_scatter_to_masses):
    // out[a][b] = sum_j (W W)[j][a] G[j][b].  Sampled bilinearly at point i this is
    // sum_j bw_i[j] ((1 - ty) G[j][b_i] + ty G[j][b_i + 1]) with the geometry-only row
    // bw_i[j] = (1 - tx) (W W)[j][a_i] + tx (W W)[j][a_i + 1].
    {
        const double *W = plan->weights;
        std::vector<double> W2((size_t)N * N, 0.0);
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++) {
                double wjk = W[(long)j * N + k];
                if (wjk == 0.0) continue;
                const double *wk = W + (long)k * N;
                double *out = W2.data() + (long)j * N;
                for (int a = 0; a < N; a++) out[a] += wjk * wk[a];
            }
        // with the secondary-axis weights folded in: w0 = (1 - ty) bw_i, w1 = ty bw_i
        for (int i = 0; i < n; i++) {
            int a = plan->back_idx[2 * i];
            double tx = plan->back_t[2 * i], ty = plan->back_t[2 * i + 1];
            double *row0 = plan->back_w + 2L * i * N;
            double *row1 = row0 + N;
            for (int j = 0; j < N; j++) {
                const double bw = (1.0 - tx) * W2[(long)j * N + a] + tx * W2[(long)j * N + a + 1];
                row0[j] = (1.0 - ty) * bw;
                row1[j] = ty * bw;
            }
        }
    }

    for (int i = 0; i < n; i++) {
        plan->pts[2 * i] = orig[i].x;
        plan->pts[2 * i + 1] = orig[i].y;
    }
    sizes->n_pts = n;
    sizes->n_tri = ntri;
    sizes->n_nbr = nnz;
    sizes->n_grid = N;
    sizes->n_levels = nlev;
    return HGB_OK;
}

}  // extern "C"
