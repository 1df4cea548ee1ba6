#include "field_io.h"

#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <memory>
#include <sstream>
#include <stdexcept>

namespace nsem_driver {

namespace {

const double PI = 3.14159265358979323846264;
const double EQUAL_EPS = 1e-7;

bool file_exists(const std::string& p) {
    std::ifstream f(p, std::ios::binary);
    return (bool)f;
}

/* token reader over the text or the binary form */
class Tokens {
public:
    virtual ~Tokens() = default;
    virtual std::string str() = 0;
    virtual double num() = 0;
    virtual uint32_t uint() = 0;
    virtual bool at_end() = 0;
};

class TextTokens : public Tokens {
public:
    TextTokens(const std::string& path) : path_(path) {
        std::ifstream in(path);
        std::stringstream ss;
        ss << in.rdbuf();
        std::string cur;
        for (char c : ss.str()) {
            if (c == '{' || c == '}' || std::isspace((unsigned char)c)) {
                if (!cur.empty()) toks_.push_back(cur);
                cur.clear();
                if (c == '{' || c == '}') toks_.push_back(std::string(1, c));
            } else {
                cur += c;
            }
        }
        if (!cur.empty()) toks_.push_back(cur);
    }
    std::string str() override {
        if (at_end()) throw std::runtime_error(path_ + ": unexpected end of file");
        return toks_[i_++];
    }
    double num() override {
        const std::string s = str();
        char* end = nullptr;
        const double v = std::strtod(s.c_str(), &end);
        if (end == s.c_str() || *end) throw std::runtime_error(path_ + ": not a number: " + s);
        return v;
    }
    uint32_t uint() override {
        const std::string s = str();
        char* end = nullptr;
        const unsigned long v = std::strtoul(s.c_str(), &end, 10);
        if (end == s.c_str() || *end) throw std::runtime_error(path_ + ": not an integer: " + s);
        return (uint32_t)v;
    }
    bool at_end() override { return i_ >= toks_.size(); }

private:
    std::string path_;
    std::vector<std::string> toks_;
    size_t i_ = 0;
};

class BinTokens : public Tokens {
public:
    BinTokens(const std::string& path) : path_(path) {
        std::ifstream in(path, std::ios::binary);
        buf_.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
    }
    std::string str() override {
        need(1);
        const size_t n = (unsigned char)buf_[pos_++];
        need(n);
        std::string s(buf_.data() + pos_, n);
        pos_ += n;
        return s;
    }
    double num() override {
        need(8);
        uint64_t u = 0;
        for (int b = 0; b < 8; b++) u |= (uint64_t)(unsigned char)buf_[pos_ + b] << (8 * b);
        pos_ += 8;
        double v;
        std::memcpy(&v, &u, 8);
        return v;
    }
    uint32_t uint() override {
        need(4);
        uint32_t u = 0;
        for (int b = 0; b < 4; b++) u |= (uint32_t)(unsigned char)buf_[pos_ + b] << (8 * b);
        pos_ += 4;
        return u;
    }
    bool at_end() override { return pos_ >= buf_.size(); }

private:
    void need(size_t n) {
        if (pos_ + n > buf_.size()) throw std::runtime_error(path_ + ": unexpected end of file");
    }
    std::string path_;
    std::vector<char> buf_;
    size_t pos_ = 0;
};

void expect(Tokens& t, const char* want, const std::string& path) {
    const std::string s = t.str();
    if (s != want) throw std::runtime_error(path + ": expected '" + want + "', found '" + s + "'");
}

bool equal_eps(double p, double q) {
    const double d = std::fabs(p - q);
    return d <= EQUAL_EPS || d <= EQUAL_EPS * std::fabs(p) || d <= EQUAL_EPS * std::fabs(q);
}

/* |(x - c) / r| as the reference's mag of a Vector */
double scaled_distance(const double* x, const double* c, const double* r) {
    const double d0 = (x[0] - c[0]) / r[0], d1 = (x[1] - c[1]) / r[1], d2 = (x[2] - c[2]) / r[2];
    return std::sqrt(d0 * d0 + (d1 * d1 + (d2 * d2 + 0.0)));
}

/* initialiser expressions (field.h:1421-1510) added to f.values */
void apply_initialiser(Tokens& t, const std::string& name, Field& f, const double* cC, long n,
                       const std::array<double, 3>& g, const std::string& path) {
    const int nc = f.ncomp;
    std::vector<double> value(nc), pert(nc);
    auto read_vals = [&](std::vector<double>& v) {
        for (int c = 0; c < nc; c++) v[c] = t.num();
    };
    if (name == "uniform") {
        read_vals(value);
        for (long i = 0; i < n; i++)
            for (int c = 0; c < nc; c++) f.values[i * nc + c] += value[c];
        return;
    }
    if (name == "cosine" || name == "cosine2" || name == "gaussian" || name == "linear") {
        read_vals(value);
        read_vals(pert);
        double center[3], radius[3];
        for (double& x : center) x = t.num();
        for (double& x : radius) x = t.num();
        const double pw = name == "cosine2" ? 2.0 : 1.0;
        for (long i = 0; i < n; i++) {
            double R = scaled_distance(cC + 3 * i, center, radius);
            for (int c = 0; c < nc; c++) {
                double val = value[c];
                if (name == "gaussian") {
                    double v = std::exp(-R * R);
                    if (equal_eps(v, 0.0)) v = 0;
                    val += pert[c] * v;
                } else {
                    const double Rc = std::fmin(1.0, R);
                    if (name == "linear") val += pert[c] * (1.0 - Rc);
                    else val += (pert[c] / 2) * std::pow(1.0 + std::cos(Rc * PI), pw);
                }
                f.values[i * nc + c] += val;
            }
        }
        return;
    }
    if (name == "gaussian-outside") {
        /* perturbation inside a sphere, gaussian decay outside it */
        read_vals(value);
        read_vals(pert);
        double center[3];
        for (double& x : center) x = t.num();
        const double radius = t.num(), radius2 = t.num();
        for (long i = 0; i < n; i++) {
            const double* x = cC + 3 * i;
            const double d0 = x[0] - center[0], d1 = x[1] - center[1], d2 = x[2] - center[2];
            double R = std::sqrt(d0 * d0 + (d1 * d1 + (d2 * d2 + 0.0)));
            R = (R - radius) / radius2;
            for (int c = 0; c < nc; c++) {
                double val = value[c];
                if (R <= 0) {
                    val += pert[c];
                } else {
                    double v = std::exp(-R * R);
                    if (equal_eps(v, 0.0)) v = 0;
                    val += pert[c] * v;
                }
                f.values[i * nc + c] += val;
            }
        }
        return;
    }
    if (name == "hydrostatic") {
        read_vals(value);
        const double scale = t.num(), expon = t.num();
        for (long i = 0; i < n; i++) {
            const double* x = cC + 3 * i;
            const double gh = x[0] * g[0] + (x[1] * g[1] + (x[2] * g[2] + 0.0));
            for (int c = 0; c < nc; c++)
                f.values[i * nc + c] += value[c] * std::pow(1.0 + scale * gh, expon);
        }
        return;
    }
    throw std::runtime_error(path + ": initialiser '" + name + "' is not supported");
}

Field read_from(Tokens& t, const std::string& path, int ncomp, const double* cC, long n_int,
                const std::array<double, 3>& g) {
    Field f;
    expect(t, "size", path);
    f.ncomp = (int)t.uint();
    if (f.ncomp != ncomp)
        throw std::runtime_error(path + ": " + std::to_string(f.ncomp) + " components, expected " +
                                 std::to_string(ncomp));
    expect(t, "internal", path);
    const uint32_t count = t.uint();
    expect(t, "{", path);
    f.values.assign((size_t)n_int * ncomp, 0.0);
    if (count <= 4) {
        for (uint32_t k = 0; k < count; k++) apply_initialiser(t, t.str(), f, cC, n_int, g, path);
    } else {
        if ((long)count != n_int)
            throw std::runtime_error(path + ": " + std::to_string(count) + " values for a mesh of " +
                                     std::to_string(n_int) + " interior nodes");
        for (size_t i = 0; i < (size_t)count * ncomp; i++) f.values[i] = t.num();
    }
    expect(t, "}", path);
    if (t.at_end()) return f;
    expect(t, "boundary", path);
    const uint32_t nb = t.uint();
    expect(t, "{", path);
    for (uint32_t k = 0; k < nb; k++) {
        BoundaryCond bc;
        bc.patch = t.str();
        expect(t, "{", path);
        while (true) {
            const std::string key = t.str();
            if (key == "}") break;
            if (key == "type") {
                bc.type = t.str();
            } else {
                /* options carry values the GPU path does not model; the
                 * binary form cannot be skipped without their types */
                bc.options.push_back(key);
                throw std::runtime_error(path + ": boundary option '" + key + "' of patch " +
                                         bc.patch + " is not supported");
            }
        }
        f.bcs.push_back(bc);
    }
    expect(t, "}", path);
    return f;
}

std::string fmt12(double v) {
    char b[40];
    std::snprintf(b, sizeof b, "%.12g", v);
    return b;
}

void put_str(std::string& out, const std::string& s) {
    std::string t;
    for (char c : s)
        if (!std::isspace((unsigned char)c)) t += c;
    if (t.empty()) return;
    out += (char)(unsigned char)t.size();
    out += t;
}

void put_u32(std::string& out, uint32_t u) {
    for (int b = 0; b < 4; b++) out += (char)((u >> (8 * b)) & 0xff);
}

void put_f64(std::string& out, double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    for (int b = 0; b < 8; b++) out += (char)((u >> (8 * b)) & 0xff);
}

}  // namespace

const BoundaryCond* Field::bc(const std::string& patch) const {
    for (const auto& b : bcs)
        if (b.patch == patch) return &b;
    return nullptr;
}

Field read_field(const std::string& base, int ncomp, const double* cC, long n_int,
                 const std::array<double, 3>& gravity, bool& found) {
    found = true;
    if (file_exists(base + ".bin")) {
        BinTokens t(base + ".bin");
        return read_from(t, base + ".bin", ncomp, cC, n_int, gravity);
    }
    if (file_exists(base + ".txt")) {
        TextTokens t(base + ".txt");
        return read_from(t, base + ".txt", ncomp, cC, n_int, gravity);
    }
    found = false;
    return Field{};
}

void write_field(const std::string& base, const Field& f, bool binary) {
    const size_t count = f.values.size() / (size_t)f.ncomp;
    if (binary) {
        std::string out;
        put_str(out, "size ");
        put_u32(out, (uint32_t)f.ncomp);
        put_str(out, "internal ");
        put_u32(out, (uint32_t)count);
        put_str(out, "\n{\n");
        for (double v : f.values) put_f64(out, v);
        put_str(out, "}\n");
        put_str(out, "boundary ");
        put_u32(out, (uint32_t)f.bcs.size());
        put_str(out, "\n{\n");
        for (const auto& b : f.bcs) {
            put_str(out, b.patch);
            put_str(out, "\n{\n");
            put_str(out, "\ttype ");
            put_str(out, b.type);
            put_str(out, "}\n");
        }
        put_str(out, "}\n");
        std::ofstream o(base + ".bin", std::ios::binary);
        if (!o) throw std::runtime_error("cannot write " + base + ".bin");
        o.write(out.data(), (std::streamsize)out.size());
        return;
    }
    std::ofstream o(base + ".txt");
    if (!o) throw std::runtime_error("cannot write " + base + ".txt");
    o << "size " << f.ncomp << "\ninternal " << count << "\n{\n";
    for (size_t i = 0; i < count; i++) {
        for (int c = 0; c < f.ncomp; c++) {
            o << fmt12(f.values[i * f.ncomp + c]);
            if (f.ncomp > 1) o << " ";
        }
        o << "\n";
    }
    o << "}\nboundary " << f.bcs.size() << "\n{\n";
    for (const auto& b : f.bcs) o << b.patch << "\n{\n\ttype " << b.type << "\n}\n";
    o << "}\n";
}

}  // namespace nsem_driver
