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
    std::array<BlockDesc::Edge, 12> edges{};
    std::array<double, 12> factor{};
    factor.fill(1.0);
    bool curved = false, wall = false;
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
            factor.fill(1.0);
            if (type == "wall" || type == "geometric") {
                /* grading factors: sz values spread over the 12 edges in
                 * groups of 12 / sz (meshApp.cpp:120-143) */
                const std::vector<double> f = c.list();
                const int sz = (int)f.size();
                if (sz < 1 || sz > 12) throw std::runtime_error(path + ": bad grading factor list");
                const int r = 12 / sz;
                for (int i = 0; i < sz; i++)
                    for (int j = 0; j < r; j++)
                        if (i * r + j < 12) factor[i * r + j] = f[i];
                for (double v : factor)
                    if (!(v > 0)) throw std::runtime_error(path + ": grading factor must be > 0");
                /* a wall-graded direction with an odd count above 1 gets one
                 * more division, and the factors of edges d, d+3, d+6, d+9
                 * are inverted (src/mesh/hexMesh.cpp:51-66, as written there) */
                if (type == "wall") {
                    wall = true;
                    for (int d = 0; d < 3; d++)
                        if (nloc[d] % 2 && nloc[d] != 1) {
                            nloc[d]++;
                            for (int i = d; i < 12; i += 3) factor[i] = 1 / factor[i];
                        }
                }
            } else if (type != "linear") {
                throw std::runtime_error(path + ": block spacing '" + type + "' is not supported");
            }
            if (!c.done() && c.peek() == "edges") {
                /* edges n{ <type> <side> <key> [scale] ... } (meshApp.cpp:159-185) */
                c.next();
                const long ne_ = c.integer();
                c.expect("{");
                for (long q = 0; q < ne_; q++) {
                    const std::string ty = c.next();
                    const long side = c.integer(), key = c.integer();
                    if (side < 0 || side >= 12 || key < 0 || key >= nkp)
                        throw std::runtime_error(path + ": edge side or key point out of range");
                    BlockDesc::Edge& ed = edges[side];
                    ed.key = kp[key];
                    if (ty == "arc") ed.type = 1;
                    else {
                        ed.scale = c.number();
                        if (ty == "cosine") ed.type = 2;
                        else if (ty == "gaussian") ed.type = 3;
                        else if (ty == "ridge") ed.type = 4;
                        else if (ty == "schar") ed.type = 5;
                        else throw std::runtime_error(path + ": edge type '" + ty + "' is not supported");
                    }
                    curved = true;
                }
                c.expect("}");
            }
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

    /* the block's own axes: v0->v1 (i), v0->v3 (j), v0->v4 (k), sides k-, k+,
     * j-, j+, i-, i+ (meshApp.cpp / hexMesh.cpp) */
    BlockDesc b;
    b.corner = corner;
    b.edge = edges;
    b.curved = curved;
    b.wall = wall;
    b.factor = factor;
    for (int a = 0; a < 3; a++) b.n[a] = nloc[a];
    const int axis_vertex[3] = {1, 3, 4};
    for (int a = 0; a < 3; a++) {
        double l = 0;
        for (int d = 0; d < 3; d++) l += std::fabs(corner[axis_vertex[a]][d] - corner[0][d]);
        if (l == 0) throw std::runtime_error(path + ": degenerate block");
    }
    static const BoxSide sides[6] = {{2, -1}, {2, 1}, {1, -1}, {1, 1}, {0, -1}, {0, 1}};
    /* block side s by its corners (hexMesh.cpp:300-312) */
    static const int side_corners[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                           {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};
    /* a patch face names the block side whose corner plane it shares: the mesh
     * app's test (meshApp.cpp:212-224), both the normals' cross product and the
     * root of the offset along the normal within 1e-3 */
    using A3 = std::array<double, 3>;
    auto sub = [](const A3& a, const A3& c2) { return A3{a[0] - c2[0], a[1] - c2[1], a[2] - c2[2]}; };
    auto crs = [](const A3& a, const A3& c2) {
        return A3{a[1] * c2[2] - a[2] * c2[1], a[2] * c2[0] - a[0] * c2[2], a[0] * c2[1] - a[1] * c2[0]};
    };
    auto dt = [](const A3& a, const A3& c2) { return a[0] * c2[0] + (a[1] * c2[1] + a[2] * c2[2]); };
    auto unit = [&](A3 a) {
        const double m = std::sqrt(dt(a, a));
        for (double& v : a) v /= m;
        return a;
    };
    auto on_side = [&](int s, const std::vector<int>& ids) -> bool {
        const A3 N = unit(crs(sub(kp[ids[1]], kp[ids[0]]), sub(kp[ids[2]], kp[ids[0]])));
        const int* sc = side_corners[s];
        const A3 pN = unit(crs(sub(corner[sc[1]], corner[sc[0]]), sub(corner[sc[2]], corner[sc[0]])));
        A3 pC;
        for (int d = 0; d < 3; d++)
            pC[d] = (corner[sc[0]][d] + corner[sc[1]][d] + corner[sc[2]][d] + corner[sc[3]][d]) / 4;
        const A3 H = unit(sub(pC, kp[ids[0]]));
        const A3 x = crs(N, pN);
        const double d1 = std::sqrt(dt(x, x));
        const double d2 = std::sqrt(std::fabs(dt(N, H)));
        return d1 <= 10e-4 && d2 <= 10e-4;
    };

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
            /* the two faces of the j or the k axis of a block one element
             * thick along it (srtb: y; advection-leveque: z) */
            const int ax = sides[s].axis;
            const int lo = ax == 1 ? 2 : 0;
            if (ax == 0 || b.patch[lo] != "delete" || b.patch[lo + 1] != "delete" || b.n[ax] != 1)
                throw std::runtime_error(path + ": only the two faces of the block's second or "
                                         "third axis, one element thick along it, can be "
                                         "deleted (2D case)");
            b.del_axis = ax;
        }
    }
    if (b.del_axis == 1) b.patch[2] = b.patch[3] = "";
    if (b.del_axis == 2) b.patch[0] = b.patch[1] = "";
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


namespace {

/* Vector arithmetic of the mesh geometry.  The operations follow the
 * reference's tensor library term by term (dot products summed from the last
 * component, src/tensor/tensor.h:124; unit vectors by division) so that the
 * geometry agrees with its LoadMesh to the last bits. */
using V3 = std::array<double, 3>;

V3 add3(const V3& a, const V3& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
V3 sub3(const V3& a, const V3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
V3 mul3(double s, const V3& a) { return {s * a[0], s * a[1], s * a[2]}; }
V3 div3(const V3& a, double s) { return {a[0] / s, a[1] / s, a[2] / s}; }
double dot3(const V3& a, const V3& b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
V3 cross3(const V3& a, const V3& b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
double mag3(const V3& a) { return std::sqrt(dot3(a, a)); }

/* block edges: vertex pairs in hex order, i-, j-, k-direction groups (meshApp.cpp:148-152) */
const int kEdgeEnds[12][2] = {{0, 1}, {3, 2}, {7, 6}, {4, 5}, {0, 3}, {1, 2},
                              {5, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

/* shape of one curved block edge (hexMesh.cpp:108-124): an arc's centre,
 * rotation axis and opening angle, or a bump's foot point and offset */
struct EdgeShape {
    int type = 0;
    V3 v0{}, v1{}, center{}, N{};
    double theta = 0, scale = 1;
};

EdgeShape edge_shape(const BlockDesc& b, int w) {
    EdgeShape e;
    const BlockDesc::Edge& ed = b.edge[w];
    e.type = ed.type;
    e.scale = ed.scale;
    e.v0 = b.corner[kEdgeEnds[w][0]];
    e.v1 = b.corner[kEdgeEnds[w][1]];
    if (e.type == 1) {
        /* circumcentre of (v0, v1, key) */
        const V3 a12 = sub3(e.v0, e.v1), a13 = sub3(e.v0, ed.key), a23 = sub3(e.v1, ed.key);
        const V3 cx = cross3(a12, a23);
        const double d = 2 * dot3(cx, cx);
        const double ca = dot3(a23, a23) * dot3(a12, a13) / d;
        const double cb = dot3(a13, a13) * dot3(mul3(-1.0, a12), a23) / d;
        const double cc = dot3(a12, a12) * dot3(a13, a23) / d;
        e.center = add3(add3(mul3(ca, e.v0), mul3(cb, e.v1)), mul3(cc, ed.key));
        const V3 r1 = sub3(e.v0, e.center), r2 = sub3(e.v1, e.center);
        e.theta = std::acos(dot3(r1, r2) / (mag3(r1) * mag3(r2)));
        const V3 N = cross3(sub3(ed.key, e.v0), sub3(e.v1, e.v0));
        e.N = div3(N, mag3(N));
    } else if (e.type != 0) {
        const V3 dd = sub3(e.v1, e.v0), pp = sub3(ed.key, e.v0);
        e.center = add3(mul3(dot3(pp, dd) / dot3(dd, dd), dd), e.v0);
        e.N = sub3(ed.key, e.center);
    }
    return e;
}

/* point at parameter m along an edge (hexMesh.cpp:20-45): straight, a
 * circular arc (v0 rotated about the arc's axis through its centre), or a
 * bump of the edge's shape towards the key point */
V3 edge_point(const EdgeShape& e, double m) {
    if (e.type == 1) {
        const V3 v = sub3(e.v0, e.center);
        const V3& N = e.N;
        const double sum = dot3(v, N), ct = std::cos(e.theta * m), st = std::sin(e.theta * m);
        V3 r;
        r[0] = N[0] * sum * (1 - ct) + v[0] * ct + (-N[2] * v[1] + N[1] * v[2]) * st;
        r[1] = N[1] * sum * (1 - ct) + v[1] * ct + (+N[2] * v[0] - N[0] * v[2]) * st;
        r[2] = N[2] * sum * (1 - ct) + v[2] * ct + (-N[1] * v[0] + N[0] * v[1]) * st;
        return add3(r, e.center);
    }
    V3 v = add3(mul3(1 - m, e.v0), mul3(m, e.v1));
    if (e.type == 0) return v;
    const double cx = mag3(sub3(e.center, e.v0)) / mag3(sub3(e.v1, e.v0));
    double mm = std::fabs(m - cx) / e.scale;
    if (e.type != 5 && mm > 0.5) mm = 0.5;
    const double PI = 3.14159265358979323846264;
    double f = 0;
    if (e.type == 2) f = std::pow(std::cos(PI * mm), 2);
    else if (e.type == 3) f = std::exp(-16 * std::pow(mm, 2));
    else if (e.type == 5) f = std::exp(-std::pow(mm, 2)) * std::pow(std::cos(PI * mm), 2);
    else if (e.type == 4) f = 1 - 2 * mm;
    return add3(v, mul3(f, e.N));
}

/* transfinite interpolation on a face from its corners and edge points
 * (the Coons patch; terms in the order of src/tensor/tensor.h:523-537) */
V3 coons_face(double r, double s, const V3& x00, const V3& x01, const V3& x10, const V3& x11,
              const V3& xr0, const V3& xr1, const V3& x0s, const V3& x1s) {
    V3 v;
    for (int q = 0; q < 3; q++)
        v[q] = -(1.0 - r) * (1.0 - s) * x00[q] + (1.0 - r) * x0s[q] - (1.0 - r) * s * x01[q] +
               (1.0 - s) * xr0[q] + s * xr1[q] - r * (1.0 - s) * x10[q] + r * x1s[q] -
               r * s * x11[q];
    return v;
}

/* transfinite interpolation in a hexahedron from its 8 corners vp (hex order),
 * the 12 edge points vd (edge order above) and the 6 face points vf (k-, k+,
 * j-, j+, i-, i+) at (r, s, t) (tensor.h:542-575, arguments as hexMesh.cpp's
 * ADDC) */
V3 coons_cell(double r, double s, double t, const V3* vp, const V3* vd, const V3* vf) {
    const V3 &x000 = vp[0], &x001 = vp[4], &x010 = vp[3], &x011 = vp[7];
    const V3 &x100 = vp[1], &x101 = vp[5], &x110 = vp[2], &x111 = vp[6];
    const V3 &xr00 = vd[0], &xr01 = vd[3], &xr10 = vd[1], &xr11 = vd[2];
    const V3 &x0s0 = vd[4], &x0s1 = vd[7], &x1s0 = vd[5], &x1s1 = vd[6];
    const V3 &x00t = vd[8], &x01t = vd[11], &x10t = vd[9], &x11t = vd[10];
    const V3 &x0st = vf[4], &x1st = vf[5], &xr0t = vf[2], &xr1t = vf[3], &xrs0 = vf[0],
             &xrs1 = vf[1];
    V3 v;
    for (int q = 0; q < 3; q++)
        v[q] = (1.0 - r) * (1.0 - s) * (1.0 - t) * x000[q] - (1.0 - r) * (1.0 - s) * x00t[q] +
               (1.0 - r) * (1.0 - s) * t * x001[q] - (1.0 - r) * (1.0 - t) * x0s0[q] +
               (1.0 - r) * x0st[q] - (1.0 - r) * t * x0s1[q] +
               (1.0 - r) * s * (1.0 - t) * x010[q] - (1.0 - r) * s * x01t[q] +
               (1.0 - r) * s * t * x011[q] - (1.0 - s) * (1.0 - t) * xr00[q] +
               (1.0 - s) * xr0t[q] - (1.0 - s) * t * xr01[q] + (1.0 - t) * xrs0[q] +
               t * xrs1[q] - s * (1.0 - t) * xr10[q] + s * xr1t[q] - s * t * xr11[q] +
               r * (1.0 - s) * (1.0 - t) * x100[q] - r * (1.0 - s) * x10t[q] +
               r * (1.0 - s) * t * x101[q] - r * (1.0 - t) * x1s0[q] + r * x1st[q] -
               r * t * x1s1[q] + r * s * (1.0 - t) * x110[q] - r * s * x11t[q] +
               r * s * t * x111[q];
    return v;
}

/* the 6 face points of a hexahedron at (r, s, t) from its corners and edge
 * points (hexMesh.cpp / dg.cpp ADDF argument lists) */
void coons_faces(double r, double s, double t, const V3* vp, const V3* vd, V3* vf) {
    vf[0] = coons_face(r, s, vp[0], vp[3], vp[1], vp[2], vd[0], vd[1], vd[4], vd[5]);
    vf[1] = coons_face(r, s, vp[4], vp[7], vp[5], vp[6], vd[3], vd[2], vd[7], vd[6]);
    vf[2] = coons_face(r, t, vp[0], vp[4], vp[1], vp[5], vd[0], vd[3], vd[8], vd[9]);
    vf[3] = coons_face(r, t, vp[3], vp[7], vp[2], vp[6], vd[1], vd[2], vd[11], vd[10]);
    vf[4] = coons_face(s, t, vp[0], vp[4], vp[3], vp[7], vd[4], vd[7], vd[8], vd[11]);
    vf[5] = coons_face(s, t, vp[1], vp[5], vp[2], vp[6], vd[5], vd[6], vd[9], vd[10]);
}

/* a node of a straight-edged hexahedron at (r, s, t) in [0, 1]^3 (dg.cpp:245-300) */
V3 hex_point(const V3* vp, double r, double s, double t) {
    V3 vd[12], vf[6];
    for (int w = 0; w < 12; w++) {
        const double m = w < 4 ? r : (w < 8 ? s : t);
        vd[w] = add3(mul3(1 - m, vp[kEdgeEnds[w][0]]), mul3(m, vp[kEdgeEnds[w][1]]));
    }
    coons_faces(r, s, t, vp, vd, vf);
    return coons_cell(r, s, t, vp, vd, vf);
}

/* the reference's equal(): within 1e-7 absolute or relative (tensor.h:471) */
bool near_equal(double p, double q) {
    const double d = std::fabs(p - q);
    return d <= 1e-7 || d <= 1e-7 * std::fabs(p) || d <= 1e-7 * std::fabs(q);
}

/* vertex parameters 0..n of a block edge with n divisions and grading factor
 * s (hexMesh.cpp:68-96): geometric progression with total ratio s, or for a
 * `wall` edge two mirrored halves each graded by s */
std::vector<double> edge_params(int n, double s, bool wall) {
    std::vector<double> sc((size_t)n + 1);
    s = wall ? std::pow(s, 1. / (n / 2.)) : std::pow(s, 1. / n);
    if (n == 1) {
        sc[0] = 0;
        sc[1] = 1;
        return sc;
    }
    const int nt = wall ? n / 2 : n;
    const double r = s;
    for (int j = 0; j <= nt; j++)
        sc[j] = near_equal(r, 1.0) ? double(j) / nt
                                   : (1 - std::pow(r, double(j))) / (1 - std::pow(s, double(nt)));
    if (wall) {
        for (int j = 0; j <= nt; j++) sc[j] /= 2;
        for (int j = 0; j <= nt; j++) sc[j + nt] = 1.0 - sc[nt - j];
    }
    return sc;
}

/* area vector of a quadrilateral mesh face as Mesh::calcGeometry forms it
 * (mesh.cpp:460-500): triangle fan about the vertex centroid, N / 2; its
 * area-weighted centre; and its vertex centroid */
void quad_area(const V3* q, V3& area, V3& centre, V3& vcentroid) {
    V3 C0 = {0, 0, 0};
    for (int j = 0; j < 4; j++) C0 = add3(C0, q[j]);
    vcentroid = div3(C0, 4.0);
    V3 N = {0, 0, 0}, C = {0, 0, 0};
    double tot = 0;
    for (int j = 0; j < 4; j++) {
        const V3& v2 = q[j];
        const V3& v3 = q[(j + 1) % 4];
        const V3 Ni = cross3(sub3(v2, vcentroid), sub3(v3, vcentroid));
        const double mn = mag3(Ni);
        C = add3(C, mul3(mn, div3(add3(add3(vcentroid, v2), v3), 3.0)));
        tot += mn;
        N = add3(N, Ni);
    }
    centre = div3(C, tot);
    area = N;  /* halved after orientation, as the reference does */
}

/* Jinv of one node from its Jacobian J[r][c] = dx_r / dxi_c: the reference's
 * pseudo-inverse ((J^T J)^-1 J^T)^T with a collapsed direction's diagonal set
 * to 1 before and 0 after the inversion (dg.cpp:412-476; tensor.cpp inv and
 * mul), stored XX YY ZZ XY YZ XZ YX ZY ZX */
void metric_pinv(const double J[3][3], const int npd[3], double out[9]) {
    double T[3][3], M[3][3], R[3][3], P[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) T[r][c] = J[c][r];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) M[r][c] = T[r][0] * J[0][c] + T[r][1] * J[1][c] + T[r][2] * J[2][c];
    for (int a = 0; a < 3; a++)
        if (npd[a] == 1) M[a][a] = 1;
    R[0][0] = M[1][1] * M[2][2] - M[1][2] * M[2][1];
    R[1][1] = M[0][0] * M[2][2] - M[0][2] * M[2][0];
    R[2][2] = M[0][0] * M[1][1] - M[0][1] * M[1][0];
    R[0][1] = M[0][2] * M[2][1] - M[0][1] * M[2][2];
    R[0][2] = M[0][1] * M[1][2] - M[0][2] * M[1][1];
    R[1][0] = M[1][2] * M[2][0] - M[1][0] * M[2][2];
    R[1][2] = M[0][2] * M[1][0] - M[0][0] * M[1][2];
    R[2][0] = M[1][0] * M[2][1] - M[1][1] * M[2][0];
    R[2][1] = M[0][1] * M[2][0] - M[0][0] * M[2][1];
    const double d = M[0][0] * R[0][0] + M[0][1] * R[1][0] + M[0][2] * R[2][0];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) R[r][c] = d == 0 ? 0.0 : R[r][c] / d;
    for (int a = 0; a < 3; a++)
        if (npd[a] == 1) R[a][a] = 0;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) P[r][c] = R[r][0] * T[0][c] + R[r][1] * T[1][c] + R[r][2] * T[2][c];
    const int order[9][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {0, 2}, {1, 0}, {2, 1}, {2, 0}};
    for (int q = 0; q < 9; q++) out[q] = P[order[q][1]][order[q][0]];
}

}  // namespace

CaseMesh build_box_mesh(const BlockDesc& b, int NPX, int NPY, int NPZ,
                        const std::array<uint32_t, 6>& side_bc) {
    if (b.del_axis == 1 && NPY != 1) throw std::runtime_error("a 2D case (y faces deleted) needs npy 0");
    if (b.del_axis == 2 && NPZ != 1) throw std::runtime_error("a 2D case (z faces deleted) needs npz 0");
    if (b.del_axis != 1 && NPY == 1) throw std::runtime_error("npy 0 needs the y faces deleted (2D case)");
    if (b.del_axis != 2 && NPZ == 1) throw std::runtime_error("npz 0 needs the z faces deleted (2D case)");
    CaseMesh M;
    const int nx = b.n[0], ny = b.del_axis == 1 ? 1 : b.n[1], nz = b.del_axis == 2 ? 1 : b.n[2];
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
    const int64_t ne = (int64_t)nx * ny * nz;
    const int lim[3] = {nx, ny, nz};
    const int64_t stride[3] = {(int64_t)ny * nz, nz, 1};
    auto coord = [&](int64_t e, int axis) -> int {
        if (axis == 0) return (int)(e / ((int64_t)ny * nz));
        if (axis == 1) return (int)((e / nz) % ny);
        return (int)(e % nz);
    };

    /* faces: interior groups normal to k, j, i (owner the lower element), then
     * the boundary sides k-, k+, j-, j+, i-, i+ with one ghost cell each */
    struct Group {
        std::vector<int64_t> own, nb, fid;
        int fo;
        bool interior;
    };
    std::vector<Group> groups;
    std::vector<int64_t> elem_faces((size_t)ne * 6, -1);
    int64_t nf = 0;
    const int inner[3][2] = {{2, 1}, {1, 3}, {0, 5}};
    for (const auto& af : inner) {
        const int axis = af[0], fo = af[1];
        if (axis == b.del_axis) continue;
        Group g;
        g.fo = fo;
        g.interior = true;
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
    for (int fo = 0; fo < 6; fo++) {
        const int axis = sides[fo].axis, sgn = sides[fo].sign;
        if (axis == b.del_axis) continue;
        Group g;
        g.fo = fo;
        g.interior = false;
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

    /* the vertex lattice by transfinite interpolation of the block's corners,
     * edges and faces (hexMesh.cpp:126-210: edge points at the edge spacing,
     * face and cell parameters i / n) */
    std::vector<V3> lat((size_t)(nx + 1) * (ny + 1) * (nz + 1));
    auto LI = [&](int i, int j, int k) -> size_t {
        return ((size_t)i * (ny + 1) + j) * (nz + 1) + k;
    };
    {
        EdgeShape es[12];
        std::vector<double> sc[12];
        const int nd[3] = {nx, ny, nz};
        for (int w = 0; w < 12; w++) {
            es[w] = edge_shape(b, w);
            sc[w] = edge_params(nd[w / 4], b.factor[w], b.wall);
        }
        const V3* cp = b.corner.data();
        for (int i = 0; i <= nx; i++)
            for (int j = 0; j <= ny; j++)
                for (int k = 0; k <= nz; k++) {
                    V3 vd[12], vf[6];
                    for (int w = 0; w < 4; w++) vd[w] = edge_point(es[w], sc[w][i]);
                    for (int w = 4; w < 8; w++) vd[w] = edge_point(es[w], sc[w][j]);
                    for (int w = 8; w < 12; w++) vd[w] = edge_point(es[w], sc[w][k]);
                    const double rx = i / double(nx), ry = j / double(ny), rz = k / double(nz);
                    coons_faces(rx, ry, rz, cp, vd, vf);
                    lat[LI(i, j, k)] = coons_cell(rx, ry, rz, cp, vd, vf);
                }
    }
    static const int bits[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    /* the 4 vertices of side fo of element e, in the mesh app's face order */
    auto face_quad = [&](int64_t e, int fo, V3* q) {
        const int axis = sides[fo].axis;
        int i0 = coord(e, 0), j0 = coord(e, 1), k0 = coord(e, 2);
        if (fo & 1) (axis == 0 ? i0 : axis == 1 ? j0 : k0)++;
        if (axis == 2) {
            q[0] = lat[LI(i0, j0, k0)]; q[1] = lat[LI(i0 + 1, j0, k0)];
            q[2] = lat[LI(i0 + 1, j0 + 1, k0)]; q[3] = lat[LI(i0, j0 + 1, k0)];
        } else if (axis == 1) {
            q[0] = lat[LI(i0, j0, k0)]; q[1] = lat[LI(i0 + 1, j0, k0)];
            q[2] = lat[LI(i0 + 1, j0, k0 + 1)]; q[3] = lat[LI(i0, j0, k0 + 1)];
        } else {
            q[0] = lat[LI(i0, j0, k0)]; q[1] = lat[LI(i0, j0 + 1, k0)];
            q[2] = lat[LI(i0, j0 + 1, k0 + 1)]; q[3] = lat[LI(i0, j0, k0 + 1)];
        }
    };

    /* element volumes and face area vectors as Mesh::calcGeometry forms them
     * (mesh.cpp:450-520): pyramids from the cell centre (the mean of its
     * faces' vertex centroids) over its 6 faces, y faces of a 2D case
     * included (LoadMesh forms them before it deletes those faces); area
     * vectors half the triangle-fan sum, pointing away from the owner */
    std::vector<double> vol_e((size_t)ne);
    std::vector<V3> cc0((size_t)ne);
    for (int64_t e = 0; e < ne; e++) {
        V3 N[6], FC[6], F0[6], q[4];
        for (int fo = 0; fo < 6; fo++) {
            face_quad(e, fo, q);
            quad_area(q, N[fo], FC[fo], F0[fo]);
        }
        V3 C = {0, 0, 0};
        for (int fo = 0; fo < 6; fo++) C = add3(C, F0[fo]);
        cc0[e] = div3(C, 6.0);
        double V = 0;
        for (int fo = 0; fo < 6; fo++) V += std::fabs(dot3(sub3(cc0[e], FC[fo]), div3(N[fo], 2.0)));
        vol_e[e] = V / 3.0;
    }
    std::vector<V3> area_f((size_t)nf);
    for (const Group& g : groups)
        for (size_t q = 0; q < g.own.size(); q++) {
            V3 qv[4], N, FC, F0;
            face_quad(g.own[q], g.fo, qv);
            quad_area(qv, N, FC, F0);
            if (dot3(sub3(FC, cc0[g.own[q]]), N) < 0) N = mul3(-1.0, N);
            area_f[g.fid[q]] = div3(N, 2.0);
        }

    /* nodes: each element straight-edged between its 8 lattice vertices, its
     * nodes by transfinite interpolation (dg.cpp:167-310), node weights
     * V_e w_i w_j w_k / 8, the metric from the LGL derivative of the node
     * coordinates (dg.cpp:412-440: the i derivative over every node of the
     * line, then the j and k derivatives' own-node term first) */
    M.cC.assign((size_t)n_all * 3, 0.0);
    M.cV.assign((size_t)n_all, 0.0);
    M.Jinv.assign((size_t)n_all * 9, 0.0);
    for (int64_t e = 0; e < ne; e++) {
        V3 vp[8];
        for (int m = 0; m < 8; m++)
            vp[m] = lat[LI(coord(e, 0) + bits[m][0], coord(e, 1) + bits[m][1], coord(e, 2) + bits[m][2])];
        for (int li = 0; li < NPX; li++)
            for (int lj = 0; lj < NPY; lj++)
                for (int lk = 0; lk < NPZ; lk++) {
                    const int64_t n = e * NP + (li * NPY + lj) * NPZ + lk;
                    const V3 x = hex_point(vp, (M.xgl[0][li] + 1) / 2, (M.xgl[1][lj] + 1) / 2,
                                           (M.xgl[2][lk] + 1) / 2);
                    for (int d = 0; d < 3; d++) M.cC[3 * n + d] = x[d];
                    M.cV[n] = vol_e[e] * (wg0[li] * wg1[lj] * wg2[lk] / 8);
                }
        auto X = [&](int i, int j, int k, int a) {
            return M.cC[3 * (e * NP + (i * NPY + j) * NPZ + k) + a];
        };
        for (int li = 0; li < NPX; li++)
            for (int lj = 0; lj < NPY; lj++)
                for (int lk = 0; lk < NPZ; lk++) {
                    const int64_t n = e * NP + (li * NPY + lj) * NPZ + lk;
                    double Jm[3][3];
                    for (int a = 0; a < 3; a++) {
                        double s0 = 0;
                        for (int i = 0; i < NPX; i++) s0 += X(i, lj, lk, a) * M.dpsi[0][li * NPX + i];
                        double s1 = X(li, lj, lk, a) * M.dpsi[1][lj * NPY + lj];
                        for (int j = 0; j < NPY; j++)
                            if (j != lj) s1 += X(li, j, lk, a) * M.dpsi[1][lj * NPY + j];
                        double s2 = X(li, lj, lk, a) * M.dpsi[2][lk * NPZ + lk];
                        for (int k = 0; k < NPZ; k++)
                            if (k != lk) s2 += X(li, lj, k, a) * M.dpsi[2][lk * NPZ + k];
                        Jm[a][0] = s0;
                        Jm[a][1] = s1;
                        Jm[a][2] = s2;
                    }
                    metric_pinv(Jm, npd, &M.Jinv[9 * n]);
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
                    for (int d = 0; d < 3; d++) M.fN[3 * k + d] = area_f[g.fid[q]][d] * w;
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
    std::vector<int> order_ids = b.del_axis == 1   ? std::vector<int>{0, 1, 4, 5}
                                 : b.del_axis == 2 ? std::vector<int>{2, 3, 4, 5}
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
