#include "case_mesh.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace nsem_driver {

namespace {

enum { XX, YY, ZZ, XY, YZ, XZ, YX, ZY, ZX };

/* tokens with `#` comments removed and braces as tokens of their own */
std::vector<std::string> read_tokens(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error("cannot open mesh description " + path);
    std::vector<std::string> out;
    std::string line;
    while (std::getline(in, line)) {
        line = line.substr(0, line.find('#'));
        std::string cur;
        for (char c : line) {
            if (c == '{' || c == '}' || std::isspace((unsigned char)c)) {
                if (!cur.empty()) out.push_back(cur);
                cur.clear();
                if (c == '{' || c == '}') out.push_back(std::string(1, c));
            } else {
                cur += c;
            }
        }
        if (!cur.empty()) out.push_back(cur);
    }
    return out;
}

struct Cursor {
    const std::vector<std::string>& t;
    const std::string& path;
    size_t i = 0;
    bool done() const { return i >= t.size(); }
    const std::string& peek() const {
        if (done()) throw std::runtime_error(path + ": unexpected end of file");
        return t[i];
    }
    std::string next() {
        const std::string s = peek();
        i++;
        return s;
    }
    void expect(const char* s) {
        const std::string w = next();
        if (w != s) throw std::runtime_error(path + ": expected '" + s + "', found '" + w + "'");
    }
    double number() {
        const std::string w = next();
        char* end = nullptr;
        const double v = std::strtod(w.c_str(), &end);
        if (end == w.c_str() || *end) throw std::runtime_error(path + ": not a number: " + w);
        return v;
    }
    long integer() {
        const std::string w = next();
        char* end = nullptr;
        const long v = std::strtol(w.c_str(), &end, 10);
        if (end == w.c_str() || *end) throw std::runtime_error(path + ": not an integer: " + w);
        return v;
    }
    /* `n{a b ...}` as the reference's IntVector / vector input */
    std::vector<double> list() {
        const long n = integer();
        expect("{");
        std::vector<double> v;
        for (long k = 0; k < n; k++) v.push_back(number());
        expect("}");
        return v;
    }
};

bool is_number_start(const std::string& s) {
    return !s.empty() && (std::isdigit((unsigned char)s[0]) || s[0] == '-' || s[0] == '+' || s[0] == '.');
}

}  // namespace

BlockDesc read_block_description(const std::string& path) {
    const std::vector<std::string> tok = read_tokens(path);
    Cursor c{tok, path};
    /* key points */
    const long nkp = c.integer();
    c.expect("{");
    std::vector<std::array<double, 3>> kp(nkp);
    for (long k = 0; k < nkp; k++)
        for (int d = 0; d < 3; d++) kp[k][d] = c.number();
    c.expect("}");

    bool have_block = false;
    std::array<std::array<double, 3>, 8> corner{};
    std::array<int, 3> nloc{};
    std::vector<std::pair<std::string, std::vector<int>>> patches;
    std::string default_name;
    while (!c.done()) {
        if (is_number_start(c.peek())) {
            if (have_block)
                throw std::runtime_error(path + ": more than one block; the driver meshes one "
                                         "axis-aligned hexahedral block");
            have_block = true;
            const std::vector<double> idx = c.list();
            if (idx.size() != 8) throw std::runtime_error(path + ": a block needs 8 key points");
            for (int m = 0; m < 8; m++) {
                const long k = (long)idx[m];
                if (k < 0 || k >= nkp) throw std::runtime_error(path + ": key point out of range");
                corner[m] = kp[k];
            }
            const std::string type = c.next();
            const std::vector<double> n = c.list();
            if (n.size() != 3) throw std::runtime_error(path + ": a block needs 3 division counts");
            for (int d = 0; d < 3; d++) {
                nloc[d] = (int)n[d];
                if (nloc[d] < 1) throw std::runtime_error(path + ": division count < 1");
            }
            if (type == "wall" || type == "geometric") {
                for (double s : c.list())
                    if (s != 1.0)
                        throw std::runtime_error(path + ": graded spacing (factor " + std::to_string(s) +
                                                 ") is not supported; uniform spacing only");
                /* a wall-graded direction with an odd count above 1 gets one
                 * more division (src/mesh/hexMesh.cpp:51-66) */
                if (type == "wall")
                    for (int d = 0; d < 3; d++)
                        if (nloc[d] % 2 && nloc[d] != 1) nloc[d]++;
            } else if (type != "linear") {
                throw std::runtime_error(path + ": block spacing '" + type + "' is not supported");
            }
            if (!c.done() && c.peek() == "edges")
                throw std::runtime_error(path + ": curved block edges are not supported");
        } else {
            const std::string name = c.next();
            if (name == "default") {
                default_name = c.next();
                continue;
            }
            bool any = false;
            while (!c.done() && is_number_start(c.peek())) {
                const std::vector<double> f = c.list();
                std::vector<int> ids;
                for (double v : f) {
                    if (v < 0 || v >= nkp) throw std::runtime_error(path + ": key point out of range");
                    ids.push_back((int)v);
                }
                if (ids.size() < 3) throw std::runtime_error(path + ": patch face needs 3+ points");
                patches.emplace_back(name, ids);
                any = true;
            }
            if (!any) throw std::runtime_error(path + ": patch " + name + " has no faces");
        }
    }
    if (!have_block) throw std::runtime_error(path + ": no block");

    /* local axes: v0->v1 (i), v0->v3 (j), v0->v4 (k), meshApp.cpp sides */
    BlockDesc b;
    const int axis_vertex[3] = {1, 3, 4};
    double scale = 0;
    for (int m = 0; m < 8; m++)
        for (int d = 0; d < 3; d++) scale = std::fmax(scale, std::fabs(corner[m][d]));
    const double tol = 1e-9 * (scale > 0 ? scale : 1.0);
    std::array<std::array<double, 3>, 3> E{};
    for (int a = 0; a < 3; a++)
        for (int d = 0; d < 3; d++) E[a][d] = corner[axis_vertex[a]][d] - corner[0][d];
    /* all corners on the parallelepiped spanned by the three edges (hex vertex order) */
    static const int bits[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    for (int m = 0; m < 8; m++)
        for (int d = 0; d < 3; d++) {
            double want = corner[0][d];
            for (int a = 0; a < 3; a++)
                if (bits[m][a]) want += E[a][d];
            if (std::fabs(corner[m][d] - want) > tol)
                throw std::runtime_error(path + ": block is not a parallelepiped "
                                         "(only straight, parallel opposite edges are supported)");
        }
    /* axis-aligned: each edge along one coordinate axis, distinct axes */
    std::array<int, 3> gaxis{};
    bool aligned = true;
    {
        std::array<bool, 3> used{};
        for (int a = 0; a < 3 && aligned; a++) {
            int g = -1, nz = 0;
            for (int d = 0; d < 3; d++)
                if (std::fabs(E[a][d]) > tol) { g = d; nz++; }
            if (nz == 0) throw std::runtime_error(path + ": degenerate block");
            if (nz != 1 || used[g]) aligned = false;
            else { used[g] = true; gaxis[a] = g; }
        }
    }
    static const BoxSide sides[6] = {{2, -1}, {2, 1}, {1, -1}, {1, 1}, {0, -1}, {0, 1}};
    /* the plane of side s: for an aligned block a coordinate; else a point and
     * the normal of the face spanned by the two other edges */
    auto on_side = [&](int s, const std::vector<int>& ids) -> bool {
        const int ax = sides[s].axis;
        if (aligned) {
            const double v = sides[s].sign < 0 ? b.lo[ax] : b.hi[ax];
            for (int id : ids)
                if (std::fabs(kp[id][ax] - v) > tol) return false;
            return true;
        }
        const auto& e1 = E[(ax + 1) % 3];
        const auto& e2 = E[(ax + 2) % 3];
        double nrm[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                         e1[0] * e2[1] - e1[1] * e2[0]};
        const double mag = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
        double P[3];
        for (int d = 0; d < 3; d++) P[d] = corner[0][d] + (sides[s].sign > 0 ? E[ax][d] : 0.0);
        for (int id : ids) {
            double dist = 0;
            for (int d = 0; d < 3; d++) dist += (kp[id][d] - P[d]) * nrm[d];
            if (std::fabs(dist) / mag > tol) return false;
        }
        return true;
    };
    if (aligned) {
        for (int d = 0; d < 3; d++) {
            b.lo[d] = corner[0][d];
            b.hi[d] = corner[0][d];
            for (int m = 0; m < 8; m++) {
                b.lo[d] = std::fmin(b.lo[d], corner[m][d]);
                b.hi[d] = std::fmax(b.hi[d], corner[m][d]);
            }
        }
        for (int a = 0; a < 3; a++) b.n[gaxis[a]] = nloc[a];
    } else {
        b.affine = true;
        b.origin = corner[0];
        b.E = E;
        for (int a = 0; a < 3; a++) b.n[a] = nloc[a];
    }

    /* patches -> block sides (a patch face selects the mesh faces in its plane,
     * meshApp.cpp:206-230) */
    for (const auto& pf : patches) {
        int found = -1;
        for (int s = 0; s < 6; s++)
            if (on_side(s, pf.second)) found = s;
        if (found < 0)
            throw std::runtime_error(path + ": patch " + pf.first + " is not on the box boundary");
        if (!b.patch[found].empty() && b.patch[found] != pf.first)
            throw std::runtime_error(path + ": box side in two patches (" + b.patch[found] + ", " +
                                     pf.first + ")");
        b.patch[found] = pf.first;
    }
    for (int s = 0; s < 6; s++)
        if (b.patch[s].empty()) b.patch[s] = default_name;
    for (int s = 0; s < 6; s++) {
        if (b.patch[s].empty())
            throw std::runtime_error(path + ": a box side belongs to no patch and no default is set");
        if (b.patch[s] == "delete") {
            if (sides[s].axis != 1 || b.patch[2] != "delete" || b.patch[3] != "delete" || b.n[1] != 1)
                throw std::runtime_error(path + ": only the two y faces of a block one element "
                                         "thick in y can be deleted (2D case)");
            b.two_d = true;
        }
    }
    if (b.two_d) b.patch[2] = b.patch[3] = "";
    return b;
}

namespace {

void legendre(int p, double x, double& L0, double& L0_1, double& L0_2) {
    double L1 = 0, L1_1 = 0, L1_2 = 0;
    L0 = 1.0;
    L0_1 = 0.0;
    L0_2 = 0.0;
    for (int i = 1; i <= p; i++) {
        const double L2 = L1, L2_1 = L1_1, L2_2 = L1_2;
        L1 = L0;
        L1_1 = L0_1;
        L1_2 = L0_2;
        const double a = (2 * i - 1.0) / i;
        const double b = (i - 1.0) / i;
        L0 = a * x * L1 - b * L2;
        L0_1 = a * (L1 + x * L1_1) - b * L2_1;
        L0_2 = a * (2 * L1_1 + x * L1_2) - b * L2_2;
    }
}

}  // namespace

void lgl(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    if (n == 1) {
        x[0] = 0.0;
        w[0] = 2.0;
        return;
    }
    const int p = n - 1, ph = n / 2;
    const double pi = 3.14159265358979323846264;
    double L0, L0_1, L0_2;
    for (int i = 0; i < ph; i++) {
        double xi = std::cos((2 * i + 1) * pi / (2 * n));
        for (int it = 0; it < 20; it++) {
            legendre(p, xi, L0, L0_1, L0_2);
            const double dx = -(1 - xi * xi) * L0_1 / (-2 * xi * L0_1 + (1 - xi * xi) * L0_2);
            xi += dx;
            if (std::fabs(dx) < 1.0e-20) break;
        }
        x[p - i] = xi;
        w[p - i] = 2 / ((double)(p * (p + 1)) * L0 * L0);
    }
    if (n != 2 * ph) {
        legendre(p, 0.0, L0, L0_1, L0_2);
        x[ph] = 0.0;
        w[ph] = 2 / ((double)(p * (p + 1)) * L0 * L0);
    }
    for (int i = 0; i < ph; i++) {
        x[i] = -x[p - i];
        w[i] = +w[p - i];
    }
}

void lagrange_tables(const std::vector<double>& xg, std::vector<double>& psi,
                     std::vector<double>& dpsi) {
    const int n = (int)xg.size();
    psi.assign((size_t)n * n, 0.0);
    dpsi.assign((size_t)n * n, 0.0);
    for (int s = 0; s < n; s++) {
        const double x = xg[s];
        for (int j = 0; j < n; j++) {
            double prod = 1.0;
            for (int k = 0; k < n; k++)
                if (k != j) prod *= (x - xg[k]) / (xg[j] - xg[k]);
            psi[j * n + s] = prod;
        }
    }
    for (int s = 0; s < n; s++) {
        const double x = xg[s];
        for (int i = 0; i < n; i++) {
            double acc = 0.0;
            for (int j = 0; j < n; j++) {
                if (i == j) continue;
                double prod = 1.0;
                for (int k = 0; k < n; k++)
                    if (k != i && k != j) prod *= (x - xg[k]) / (xg[i] - xg[k]);
                acc += prod / (xg[i] - xg[j]);
            }
            dpsi[s * n + i] = acc;
        }
    }
}

CaseMesh build_box_mesh(const BlockDesc& b, int NPX, int NPY, int NPZ,
                        const std::array<uint32_t, 6>& side_bc) {
    if (b.two_d && NPY != 1) throw std::runtime_error("a 2D case (y faces deleted) needs npy 0");
    if (!b.two_d && NPY == 1) throw std::runtime_error("npy 0 needs the y faces deleted (2D case)");
    CaseMesh M;
    const int nx = b.n[0], ny = b.two_d ? 1 : b.n[1], nz = b.n[2];
    const int NP = NPX * NPY * NPZ;
    int NPF;
    if (NPX <= NPY && NPX <= NPZ) NPF = NPY * NPZ;
    else if (NPY <= NPX && NPY <= NPZ) NPF = NPX * NPZ;
    else NPF = NPX * NPY;
    M.npx = NPX; M.npy = NPY; M.npz = NPZ; M.np = NP; M.npf = NPF;
    const int npd[3] = {NPX, NPY, NPZ};
    for (int d = 0; d < 3; d++) {
        lgl(npd[d], M.xgl[d], M.wgl[d]);
        lagrange_tables(M.xgl[d], M.psi[d], M.dpsi[d]);
    }
    const auto& wg0 = M.wgl[0];
    const auto& wg1 = M.wgl[1];
    const auto& wg2 = M.wgl[2];
    const double hx = (b.hi[0] - b.lo[0]) / nx, hy = (b.hi[1] - b.lo[1]) / ny,
                 hz = (b.hi[2] - b.lo[2]) / nz;
    const int64_t ne = (int64_t)nx * ny * nz;
    const int lim[3] = {nx, ny, nz};
    const int64_t stride[3] = {(int64_t)ny * nz, nz, 1};
    auto coord = [&](int64_t e, int axis) -> int {
        if (axis == 0) return (int)(e / ((int64_t)ny * nz));
        if (axis == 1) return (int)((e / nz) % ny);
        return (int)(e % nz);
    };
    const double area[3] = {hy * hz, hx * hz, hx * hy};

    /* non-axis-aligned block: element edge vectors e_a = E_a / n_a and the
     * area vectors e_{a+1} x e_{a+2} of the faces normal to axis a, along +e_a */
    double ev[3][3] = {}, AV[3][3] = {};
    if (b.affine) {
        for (int a = 0; a < 3; a++)
            for (int d = 0; d < 3; d++) ev[a][d] = b.E[a][d] / lim[a];
        for (int a = 0; a < 3; a++) {
            const double* e1 = ev[(a + 1) % 3];
            const double* e2 = ev[(a + 2) % 3];
            AV[a][0] = e1[1] * e2[2] - e1[2] * e2[1];
            AV[a][1] = e1[2] * e2[0] - e1[0] * e2[2];
            AV[a][2] = e1[0] * e2[1] - e1[1] * e2[0];
            const double dot = AV[a][0] * ev[a][0] + AV[a][1] * ev[a][1] + AV[a][2] * ev[a][2];
            if (dot < 0)
                for (int d = 0; d < 3; d++) AV[a][d] = -AV[a][d];
        }
    }

    struct Group {
        std::vector<int64_t> own, nb, fid;
        int fo;
        double nv[3];
        bool interior;
    };
    std::vector<Group> groups;
    std::vector<int64_t> elem_faces((size_t)ne * 6, -1);
    int64_t nf = 0;
    const int inner[3][2] = {{2, 1}, {1, 3}, {0, 5}};
    for (const auto& af : inner) {
        const int axis = af[0], fo = af[1];
        if (b.two_d && axis == 1) continue;
        Group g;
        g.fo = fo;
        g.interior = true;
        g.nv[0] = g.nv[1] = g.nv[2] = 0.0;
        g.nv[axis] = area[axis];
        if (b.affine)
            for (int d = 0; d < 3; d++) g.nv[d] = AV[axis][d];
        for (int64_t e = 0; e < ne; e++)
            if (coord(e, axis) < lim[axis] - 1) {
                g.own.push_back(e);
                g.nb.push_back(e + stride[axis]);
                g.fid.push_back(nf);
                elem_faces[e * 6 + fo] = nf;
                elem_faces[(e + stride[axis]) * 6 + fo - 1] = nf;
                nf++;
            }
        groups.push_back(g);
    }
    static const BoxSide sides[6] = {{2, -1}, {2, 1}, {1, -1}, {1, 1}, {0, -1}, {0, 1}};
    int64_t n_bf = 0;
    std::vector<int64_t> bfaces;
    std::vector<int> group_side;
    for (int fo = 0; fo < 6; fo++) {
        const int axis = sides[fo].axis, sgn = sides[fo].sign;
        if (b.two_d && axis == 1) continue;
        Group g;
        g.fo = fo;
        g.interior = false;
        g.nv[0] = g.nv[1] = g.nv[2] = 0.0;
        g.nv[axis] = sgn * area[axis];
        if (b.affine)
            for (int d = 0; d < 3; d++) g.nv[d] = sgn * AV[axis][d];
        for (int64_t e = 0; e < ne; e++)
            if (coord(e, axis) == (sgn < 0 ? 0 : lim[axis] - 1)) {
                g.own.push_back(e);
                g.nb.push_back(ne + n_bf);
                g.fid.push_back(nf);
                elem_faces[e * 6 + fo] = nf;
                bfaces.push_back(nf);
                nf++;
                n_bf++;
            }
        groups.push_back(g);
    }
    const int64_t n_cells = ne + n_bf, n_int = ne * NP, n_all = n_cells * NP;
    M.n_elem = ne; M.n_cells = n_cells; M.n_face = nf; M.n_int = n_int; M.n_all = n_all;

    /* node coordinates, weights, metric */
    M.cC.assign((size_t)n_all * 3, 0.0);
    M.cV.assign((size_t)n_all, 0.0);
    M.Jinv.assign((size_t)n_all * 9, 0.0);
    double V = hx * hy * hz;
    double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    J[XX] = NPX > 1 ? 2.0 / hx : 0.0;
    J[YY] = NPY > 1 ? 2.0 / hy : 0.0;
    J[ZZ] = NPZ > 1 ? 2.0 / hz : 0.0;
    if (b.affine) {
        /* V_e = |det(e_0, e_1, e_2)|; Jinv as dg.cpp:412-476 forms it from the
         * Jacobian dx/dxi (columns e_a / 2 on the reference cube [-1, 1]^3, zero
         * for a direction with one node): ((J^T J)^-1 J^T)^T with the collapsed
         * diagonal set to 1 before and 0 after the inversion */
        V = std::fabs(ev[0][0] * AV[0][0] + ev[0][1] * AV[0][1] + ev[0][2] * AV[0][2]);
        double Jm[3][3];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) Jm[r][c] = npd[c] > 1 ? ev[c][r] / 2 : 0.0;
        double Mm[3][3];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++)
                Mm[r][c] = Jm[0][r] * Jm[0][c] + Jm[1][r] * Jm[1][c] + Jm[2][r] * Jm[2][c];
        for (int a = 0; a < 3; a++)
            if (npd[a] == 1) Mm[a][a] = 1;
        const double det = Mm[0][0] * (Mm[1][1] * Mm[2][2] - Mm[1][2] * Mm[2][1]) -
                           Mm[0][1] * (Mm[1][0] * Mm[2][2] - Mm[1][2] * Mm[2][0]) +
                           Mm[0][2] * (Mm[1][0] * Mm[2][1] - Mm[1][1] * Mm[2][0]);
        double Mi[3][3];
        Mi[0][0] = (Mm[1][1] * Mm[2][2] - Mm[1][2] * Mm[2][1]) / det;
        Mi[0][1] = (Mm[0][2] * Mm[2][1] - Mm[0][1] * Mm[2][2]) / det;
        Mi[0][2] = (Mm[0][1] * Mm[1][2] - Mm[0][2] * Mm[1][1]) / det;
        Mi[1][0] = (Mm[1][2] * Mm[2][0] - Mm[1][0] * Mm[2][2]) / det;
        Mi[1][1] = (Mm[0][0] * Mm[2][2] - Mm[0][2] * Mm[2][0]) / det;
        Mi[1][2] = (Mm[0][2] * Mm[1][0] - Mm[0][0] * Mm[1][2]) / det;
        Mi[2][0] = (Mm[1][0] * Mm[2][1] - Mm[1][1] * Mm[2][0]) / det;
        Mi[2][1] = (Mm[0][1] * Mm[2][0] - Mm[0][0] * Mm[2][1]) / det;
        Mi[2][2] = (Mm[0][0] * Mm[1][1] - Mm[0][1] * Mm[1][0]) / det;
        for (int a = 0; a < 3; a++)
            if (npd[a] == 1) Mi[a][a] = 0;
        /* P = Mi J^T (3 x 3), Jinv = P^T: Jinv[r][c] = P[c][r] */
        double P[3][3];
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++)
                P[r][c] = Mi[r][0] * Jm[c][0] + Mi[r][1] * Jm[c][1] + Mi[r][2] * Jm[c][2];
        const int order[9][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {0, 2}, {1, 0}, {2, 1}, {2, 0}};
        for (int q = 0; q < 9; q++) J[q] = P[order[q][1]][order[q][0]];
    }
    for (int64_t e = 0; e < ne; e++) {
        const int ix = coord(e, 0), iy = coord(e, 1), iz = coord(e, 2);
        for (int li = 0; li < NPX; li++)
            for (int lj = 0; lj < NPY; lj++)
                for (int lk = 0; lk < NPZ; lk++) {
                    const int t = (li * NPY + lj) * NPZ + lk;
                    const int64_t n = e * NP + t;
                    const double rx = (M.xgl[0][li] + 1) / 2, ry = (M.xgl[1][lj] + 1) / 2,
                                 rz = (M.xgl[2][lk] + 1) / 2;
                    if (b.affine) {
                        for (int d = 0; d < 3; d++)
                            M.cC[3 * n + d] = b.origin[d] + ((ix + rx) * ev[0][d] +
                                                             ((iy + ry) * ev[1][d] + (iz + rz) * ev[2][d]));
                    } else {
                        M.cC[3 * n + 0] = b.lo[0] + (ix * hx + rx * hx);
                        M.cC[3 * n + 1] = b.lo[1] + (iy * hy + ry * hy);
                        M.cC[3 * n + 2] = b.lo[2] + (iz * hz + rz * hz);
                    }
                    M.cV[n] = V * (wg0[li] * wg1[lj] * wg2[lk] / 8);
                    for (int c = 0; c < 9; c++) M.Jinv[9 * n + c] = J[c];
                }
    }

    /* face slots (dg.cpp:323-410) */
    const uint32_t sentinel = (uint32_t)n_all;
    M.FO.assign((size_t)nf * NPF, sentinel);
    M.FN.assign((size_t)nf * NPF, sentinel);
    M.fN.assign((size_t)nf * NPF * 3, 0.0);
    M.fI.assign((size_t)nf * NPF, 0.0);
    M.bc_U.assign((size_t)nf * NPF, 0u);
    M.slot_side.assign((size_t)nf * NPF, -1);
    const int face_map[6] = {0, NPZ - 1, 0, NPY - 1, 0, NPX - 1};
    auto local = [&](int fo, int a, int bb, int v) -> int {
        if (fo == 0 || fo == 1) return a * NPY * NPZ + bb * NPZ + v;
        if (fo == 2 || fo == 3) return a * NPY * NPZ + v * NPZ + bb;
        return v * NPY * NPZ + a * NPZ + bb;
    };
    for (const Group& g : groups) {
        const int fo = g.fo, vo = face_map[fo], vn = face_map[fo ^ 1];
        int ra, rb;
        const std::vector<double>*wa, *wb;
        if (fo == 0 || fo == 1) { ra = NPX; rb = NPY; wa = &wg0; wb = &wg1; }
        else if (fo == 2 || fo == 3) { ra = NPX; rb = NPZ; wa = &wg0; wb = &wg2; }
        else { ra = NPY; rb = NPZ; wa = &wg1; wb = &wg2; }
        for (size_t q = 0; q < g.own.size(); q++)
            for (int A = 0; A < ra; A++)
                for (int B = 0; B < rb; B++) {
                    const int64_t k = g.fid[q] * NPF + (A * rb + B);
                    const int64_t o = g.own[q] * NP + local(fo, A, B, vo);
                    const int64_t nn = g.nb[q] * NP + local(fo, A, B, vn);
                    const double w = (*wa)[A] * (*wb)[B] / 4;
                    M.FO[k] = (uint32_t)o;
                    M.FN[k] = (uint32_t)nn;
                    for (int d = 0; d < 3; d++) M.fN[3 * k + d] = g.nv[d] * w;
                    if (g.interior) {
                        M.fI[k] = 0.5;
                    } else {
                        M.bc_U[k] = side_bc[fo];
                        M.slot_side[k] = (int8_t)fo;
                        for (int d = 0; d < 3; d++) M.cC[3 * nn + d] = M.cC[3 * o + d];
                        M.cV[nn] = M.cV[o];
                    }
                }
    }

    /* cell face lists (interior: z-, z+, y-, y+, x-, x+; ghost: its face) */
    std::vector<int> order_ids = b.two_d ? std::vector<int>{0, 1, 4, 5}
                                         : std::vector<int>{0, 1, 2, 3, 4, 5};
    const int nfe = (int)order_ids.size();
    for (int64_t e = 0; e < ne; e++)
        for (int f : order_ids) M.all_faces.push_back((uint32_t)elem_faces[e * 6 + f]);
    for (int64_t f : bfaces) M.all_faces.push_back((uint32_t)f);
    M.face_idx0.resize((size_t)n_cells);
    M.face_idx1.resize((size_t)n_cells);
    for (int64_t e = 0; e < ne; e++) {
        M.face_idx0[e] = (uint32_t)(e * nfe);
        M.face_idx1[e] = (uint32_t)(e * nfe + nfe);
    }
    for (int64_t q = 0; q < n_bf; q++) {
        M.face_idx0[ne + q] = (uint32_t)(ne * nfe + q);
        M.face_idx1[ne + q] = (uint32_t)(ne * nfe + q + 1);
    }
    return M;
}

nsem_mesh_desc CaseMesh::desc() const {
    nsem_mesh_desc d{};
    d.npx = npx; d.npy = npy; d.npz = npz; d.npf = npf;
    d.n_elem = (int32_t)n_elem;
    d.n_cells = (int32_t)n_cells;
    d.n_face = (int32_t)n_face;
    d.cC = cC.data(); d.cV = cV.data(); d.Jinv = Jinv.data();
    d.FO = FO.data(); d.FN = FN.data(); d.fN = fN.data(); d.fI = fI.data();
    d.all_faces = all_faces.data();
    d.face_idx0 = face_idx0.data();
    d.face_idx1 = face_idx1.data();
    for (int k = 0; k < 3; k++) {
        d.psi[k] = psi[k].data();
        d.dpsi[k] = dpsi[k].data();
    }
    d.bc_U = bc_U.data();
    return d;
}

}  // namespace nsem_driver
