/*
 * nsem_euler -- the euler app's control-file-driven time loop on the GPU.
 *
 * Drop-in host driver for apps/euler/euler.cpp (and the scalar
 * apps/convection/convection.cpp): run from a case directory as the
 * reference is run,
 *
 *     nsem_euler ./controls [--scheme ref|ssprk3] [--prec fp64|mixed]
 *                           [--print-every K] [--device D] [--blocks FILE] [--dump DIR]
 *
 * It reads the controls file, the block description (the mesh app's input:
 * --blocks, by default the file named by the controls' `mesh` key), and
 * the fields p, U, T, rho at start_step / write_interval; sets up the
 * hydrostatic background and rho from p as euler.cpp:104-147 does; advances
 * the state through libnsem_gpu's C ABI; prints the mass / energy / volume
 * losses as euler.cpp:263-279; and writes rho, U, T, p every write_interval
 * steps as Iteration::next does (src/solvers/iteration.h:62-84).
 *
 * --scheme ref (default) is the reference's own update (segregated forward
 * Euler, time_scheme BDF1 or AB1, which perform the same arithmetic);
 * --scheme ssprk3 the coupled SSP-RK3 of the same operators, in FP64 or the
 * precision form (--prec mixed).  --dump writes the mesh arrays and the
 * initial fields as raw little-endian files and exits without using a GPU.
 * Options the GPU path does not model (other boundary conditions, flux or
 * time schemes, multi-block meshes, steady state, adaptive refinement) are
 * refused with a message; there is no CPU fallback.
 */
#include <sys/stat.h>

#include <algorithm>
#include <array>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "case_mesh.h"
#include "controls.h"
#include "field_io.h"
#include "nsem.h"

using namespace nsem_driver;

namespace {

struct Options {
    std::string controls;
    std::string scheme = "ref";
    std::string prec = "fp64";
    long print_every = 1;
    int device = 0;
    std::string dump;
    std::string blocks;
};

[[noreturn]] void usage(const char* msg) {
    if (msg) std::fprintf(stderr, "nsem_euler: %s\n", msg);
    std::fprintf(stderr,
                 "usage: nsem_euler <controls> [--scheme ref|ssprk3] [--prec fp64|mixed]\n"
                 "                  [--print-every K] [--device D] [--blocks FILE] [--dump DIR]\n");
    std::exit(2);
}

Options parse_args(int argc, char** argv) {
    Options o;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        auto val = [&]() -> std::string {
            if (i + 1 >= argc) usage(("missing value after " + a).c_str());
            return argv[++i];
        };
        if (a == "--scheme") o.scheme = val();
        else if (a == "--prec") o.prec = val();
        else if (a == "--print-every") o.print_every = std::atol(val().c_str());
        else if (a == "--device") o.device = std::atoi(val().c_str());
        else if (a == "--dump") o.dump = val();
        else if (a == "--blocks") o.blocks = val();
        else if (a == "-h" || a == "--help") usage(nullptr);
        else if (!a.empty() && a[0] == '-') usage(("unknown option " + a).c_str());
        else if (o.controls.empty()) o.controls = a;
        else usage("more than one controls file");
    }
    if (o.controls.empty()) usage("no controls file");
    if (o.scheme != "ref" && o.scheme != "ssprk3") usage("--scheme is ref or ssprk3");
    if (o.prec != "fp64" && o.prec != "mixed") usage("--prec is fp64 or mixed");
    if (o.scheme == "ref" && o.prec != "fp64") usage("the reference's scheme runs in FP64 only");
    if (o.print_every < 1) usage("--print-every must be >= 1");
    return o;
}

void check(nsem_ctx* ctx, nsem_status s, const char* what) {
    if (s == NSEM_OK) return;
    throw std::runtime_error(std::string(what) + " failed (status " + std::to_string((int)s) +
                             "): " + (ctx ? nsem_last_error(ctx) : ""));
}

std::string upper(std::string s) {
    for (auto& c : s) c = (char)std::toupper((unsigned char)c);
    return s;
}

template <typename T>
void dump_raw(const std::string& dir, const std::string& name, const std::vector<T>& v,
              const char* ext) {
    std::ofstream o(dir + "/" + name + ext, std::ios::binary);
    if (!o) throw std::runtime_error("cannot write " + dir + "/" + name + ext);
    o.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

/* boundary condition codes of the six box sides for the velocity field and
 * the check that scalar fields are NEUMANN wherever a patch exists */
std::array<uint32_t, 6> side_conditions(const BlockDesc& b, const Field& U,
                                        const std::vector<std::pair<std::string, const Field*>>& scalars) {
    std::array<uint32_t, 6> bc{};
    for (int s = 0; s < 6; s++) {
        const std::string& patch = b.patch[s];
        if (patch.empty()) continue;   /* deleted (2D) */
        const BoundaryCond* u = U.bc(patch);
        if (!u) throw std::runtime_error("field U has no boundary condition for patch " + patch);
        const std::string t = upper(u->type);
        if (t == "NEUMANN") bc[s] = 1;
        else if (t == "SYMMETRY") bc[s] = 2;
        else
            throw std::runtime_error("boundary condition " + u->type + " of U on patch " + patch +
                                     " is not supported (NEUMANN or SYMMETRY)");
        for (const auto& sf : scalars) {
            if (!sf.second) continue;
            const BoundaryCond* c = sf.second->bc(patch);
            if (!c) throw std::runtime_error("field " + sf.first + " has no boundary condition for patch " + patch);
            if (upper(c->type) != "NEUMANN")
                throw std::runtime_error("boundary condition " + c->type + " of " + sf.first +
                                         " on patch " + patch + " is not supported (NEUMANN)");
        }
    }
    return bc;
}

int run(const Options& opt) {
    const Controls ctl(opt.controls);
    const std::string solver = ctl.str("general", "solver", "euler");
    if (solver != "euler" && solver != "convection")
        throw std::runtime_error("solver " + solver + " is not the euler or convection app");
    const bool conv = solver == "convection";

    /* Controls:: and Fluid:: (src/field/field.cpp:51-75, apps/utils/properties.cpp) */
    const double P0 = ctl.num("general", "P0", 101325), T0 = ctl.num("general", "T0", 300);
    const double cp = ctl.num("general", "cp", 1004.67), cv = ctl.num("general", "cv", 715.5);
    const double viscosity = ctl.num("general", "viscosity", 1.568e-5), Pr = ctl.num("general", "Pr", 0.9);
    const double dt = ctl.num("general", "dt", 0.1);
    const long start_step = ctl.integer("general", "start_step", 0);
    const long end_step = ctl.integer("general", "end_step", 2);
    const long write_interval = ctl.integer("general", "write_interval", 20);
    const std::vector<double> gv = ctl.vec("general", "gravity", 3, {0, 0, -9.860616});
    const std::string mesh_name = ctl.str("general", "mesh", "grid");
    const bool binary = upper(ctl.str("general", "write_format", "BINARY")) != "TEXT";
    if (upper(ctl.str("general", "state", "STEADY")) != "TRANSIENT")
        throw std::runtime_error("state must be TRANSIENT (the steady-state relaxation is not modelled)");
    if (upper(ctl.str("general", "convection_scheme", "HYBRID")) != "RUSANOV")
        throw std::runtime_error("convection_scheme must be RUSANOV (the DG flux of the GPU path)");
    const std::string ts = upper(ctl.str("general", "time_scheme", "BDF1"));
    if (opt.scheme == "ref" && ts != "BDF1" && ts != "AB1" && !(conv && ts == "AB2"))
        throw std::runtime_error("time_scheme " + ts + " is not supported (BDF1 or AB1; AB2 for "
                                 "the convection app)");
    const int conv_order = ts == "AB2" ? 2 : 1;
    if (ctl.integer("general", "n_deferred", 0) != 0)
        throw std::runtime_error("n_deferred must be 0");
    if (write_interval < 1) throw std::runtime_error("write_interval must be >= 1");
    if (ctl.integer("general", "amr_step", 0) != 0)
        throw std::runtime_error("amr_step is set: adaptive mesh refinement is not supported");
    const std::string app = conv ? "convection" : "euler";
    const std::string pinit = upper(ctl.str(app, "problem_init", "NONE"));
    /* the convection app's analytic winds: LEVEQUE on flat meshes
     * (convection.cpp:86-91); the LAURITZEN winds need the spherical meshes */
    const bool leveque = conv && pinit == "LEVEQUE";
    if (pinit != "NONE" && !leveque)
        throw std::runtime_error("problem_init must be NONE (or LEVEQUE for the convection app)");
    const bool buoyancy = conv ? false : ctl.flag("euler", "buoyancy", true);
    const bool diffusion = conv ? false : ctl.flag("euler", "diffusion", true);
    const int npx = (int)ctl.integer("general", "npx", 1) + 1;
    const int npy = (int)ctl.integer("general", "npy", 1) + 1;
    const int npz = (int)ctl.integer("general", "npz", 1) + 1;
    if (npx < 1 || npy < 1 || npz < 1 || npx > 10 || npy > 10 || npz > 10)
        throw std::runtime_error("npx/npy/npz out of range (0..9)");

    /* mesh: the block description the mesh app reads (the reference's
     * test.sh runs `mesh <file> -o <mesh>_0.bin`); by default a file named
     * after the controls' mesh key */
    const std::string blocks = opt.blocks.empty() ? mesh_name : opt.blocks;
    {
        std::ifstream probe(blocks);
        if (!probe)
            throw std::runtime_error("no block description '" + blocks +
                                     "' (the mesh app's input file; name it with --blocks)");
    }
    const BlockDesc blk = read_block_description(blocks);
    /* node coordinates first (boundary conditions fill bc_U below) */
    CaseMesh M = build_box_mesh(blk, npx, npy, npz, {1, 1, 1, 1, 1, 1});
    const long n = (long)M.n_int;
    const std::array<double, 3> g = {gv[0], gv[1], gv[2]};

    /* fields at start_step (Iteration, iteration.h:18-40) */
    const long index = start_step / write_interval;
    const std::string sfx = std::to_string(index);
    bool fU, fT, fp = false, fr = false;
    Field U = read_field("U" + sfx, 3, M.cC.data(), n, g, fU);
    Field T = read_field("T" + sfx, 1, M.cC.data(), n, g, fT);
    if (!fU || !fT) throw std::runtime_error("fields U" + sfx + " and T" + sfx + " are required");
    Field p, rho;
    if (!conv) {
        p = read_field("p" + sfx, 1, M.cC.data(), n, g, fp);
        rho = read_field("rho" + sfx, 1, M.cC.data(), n, g, fr);
        if (!fp) throw std::runtime_error("field p" + sfx + " is required");
    }
    std::vector<std::pair<std::string, const Field*>> scalars = {{"T", &T}};
    if (!conv) {
        scalars.push_back({"p", &p});
        if (fr) scalars.push_back({"rho", &rho});
    }
    const std::array<uint32_t, 6> side_bc = side_conditions(blk, U, scalars);
    for (size_t k = 0; k < M.bc_U.size(); k++)
        if (M.slot_side[k] >= 0) M.bc_U[k] = side_bc[M.slot_side[k]];

    /* hydrostatic background and rho from p (euler.cpp:104-147) */
    const double R = cp - cv, gam = cp / cv;
    const double gb[3] = {buoyancy ? g[0] : 0.0, buoyancy ? g[1] : 0.0, buoyancy ? g[2] : 0.0};
    const int64_t n_all = M.n_all;
    std::vector<double> p_ref(n_all), rho_ref(n_all);
    for (int64_t i = 0; i < n_all; i++) {
        if (buoyancy) {
            const double* x = &M.cC[3 * i];
            const double gh = x[0] * gb[0] + (x[1] * gb[1] + (x[2] * gb[2] + 0.0));
            p_ref[i] = P0 * std::pow(1.0 + gh / (cp * T0), cp / R);
            rho_ref[i] = (P0 / (R * T0)) * std::pow(p_ref[i] / P0, 1 / gam);
        } else {
            p_ref[i] = P0;
            rho_ref[i] = P0 / (R * T0);
        }
    }
    std::vector<double> rho0(n);
    if (!conv)
        for (long i = 0; i < n; i++) {
            const double pf = p.values[i] + p_ref[i];
            rho0[i] = (P0 / (R * (T.values[i] + T0))) * std::pow(pf / P0, 1 / gam);
        }

    const nsem_mesh_desc desc = M.desc();
    if (!opt.dump.empty()) {
        mkdir(opt.dump.c_str(), 0755);
        std::vector<uint32_t> meta(16, 0);
        const uint32_t mv[11] = {(uint32_t)M.npx, (uint32_t)M.npy, (uint32_t)M.npz, (uint32_t)M.np,
                                 (uint32_t)M.npf, (uint32_t)M.n_elem, (uint32_t)M.n_cells,
                                 (uint32_t)M.n_int, (uint32_t)M.n_all, (uint32_t)M.n_face,
                                 (uint32_t)M.all_faces.size()};
        for (int k = 0; k < 11; k++) meta[k] = mv[k];
        dump_raw(opt.dump, "meta", meta, ".u32");
        dump_raw(opt.dump, "cC", M.cC, ".f64");
        dump_raw(opt.dump, "cV", M.cV, ".f64");
        dump_raw(opt.dump, "Jinv", M.Jinv, ".f64");
        dump_raw(opt.dump, "fN", M.fN, ".f64");
        dump_raw(opt.dump, "fI", M.fI, ".f64");
        dump_raw(opt.dump, "FO", M.FO, ".u32");
        dump_raw(opt.dump, "FN", M.FN, ".u32");
        dump_raw(opt.dump, "allFaces", M.all_faces, ".u32");
        dump_raw(opt.dump, "faceIdx0", M.face_idx0, ".u32");
        dump_raw(opt.dump, "faceIdx1", M.face_idx1, ".u32");
        dump_raw(opt.dump, "bcU", M.bc_U, ".u32");
        for (int d = 0; d < 3; d++) {
            const std::string s = std::to_string(d);
            dump_raw(opt.dump, "xgl" + s, M.xgl[d], ".f64");
            dump_raw(opt.dump, "wgl" + s, M.wgl[d], ".f64");
            dump_raw(opt.dump, "psi" + s, M.psi[d], ".f64");
            dump_raw(opt.dump, "dpsi" + s, M.dpsi[d], ".f64");
        }
        dump_raw(opt.dump, "p_ref", p_ref, ".f64");
        dump_raw(opt.dump, "rho_ref", rho_ref, ".f64");
        dump_raw(opt.dump, "fld_U", U.values, ".f64");
        dump_raw(opt.dump, "fld_T", T.values, ".f64");
        if (!conv) dump_raw(opt.dump, "fld_rho", rho0, ".f64");
        /* the step-0 fields in the reference's binary field format, as the
         * solver writes them */
        write_field(opt.dump + "/U0", U, true);
        write_field(opt.dump + "/T0", T, true);
        if (!conv) {
            Field r;
            r.values = rho0;
            r.bcs = fr ? rho.bcs : p.bcs;
            write_field(opt.dump + "/rho0", r, true);
        }
        std::printf("nsem_euler: wrote the case arrays to %s\n", opt.dump.c_str());
        return 0;
    }

    nsem_params prm{};
    prm.P0 = P0; prm.T0 = T0; prm.cp = cp; prm.cv = cv;
    for (int d = 0; d < 3; d++) prm.gravity[d] = gb[d];
    prm.dt = dt;
    prm.p_ref = p_ref.data();
    prm.rho_ref = rho_ref.data();
    prm.device = opt.device;
    prm.viscosity = diffusion ? viscosity : 0.0;
    prm.Pr = Pr;
    nsem_ctx* ctx = nullptr;
    check(ctx, nsem_create(&desc, &prm, &ctx), "nsem_create");
    struct Guard {
        nsem_ctx* c;
        ~Guard() { nsem_destroy(c); }
    } guard{ctx};

    std::printf("--------------------------------------------\n");
    std::printf("nsem_euler: %s, %ld elements, N = (%d, %d, %d), %ld interior nodes, %s %s\n",
                solver.c_str(), (long)M.n_elem, npx - 1, npy - 1, npz - 1, n,
                conv ? "BDF1" : (opt.scheme == "ref" ? ts.c_str() : "SSP-RK3"),
                opt.prec == "mixed" ? "precision form" : "FP64");
    const nsem_scheme scheme = opt.scheme == "ref" ? NSEM_REF_SEGREGATED : NSEM_SSPRK3;
    const nsem_precision prec = opt.prec == "mixed" ? NSEM_MIXED : NSEM_FP64;

    /* the gravity field of a buoyant run (euler.cpp:103-110: uniform g with the
     * velocity's patches as CALC_DIRICHLET), written with the other fields */
    auto write_gravity = [&](const std::string& s) {
        if (!buoyancy) return;
        Field gf;
        gf.ncomp = 3;
        gf.values.resize((size_t)n * 3);
        for (long k = 0; k < n; k++)
            for (int d = 0; d < 3; d++) gf.values[3 * k + d] = g[d];
        gf.bcs = U.bcs;
        for (auto& b : gf.bcs) b.type = "CALC_DIRICHLET";
        write_field("gravity" + s, gf, binary);
    };
    auto write_all = [&](long step) {
        const std::string s = std::to_string(step / write_interval);
        if (conv) {
            Field t = T;
            check(ctx, nsem_convection_get(ctx, t.values.data()), "nsem_convection_get");
            write_field("T" + s, t, binary);
            return;
        }
        Field r = rho, u = U, t = T, pp = p;
        if (!fr) {
            r.ncomp = 1;
            r.bcs = p.bcs;
        }
        r.values.assign(n, 0.0);
        check(ctx, nsem_get_fields(ctx, r.values.data(), u.values.data(), t.values.data()),
              "nsem_get_fields");
        check(ctx, nsem_get_pressure(ctx, pp.values.data()), "nsem_get_pressure");
        write_field("rho" + s, r, binary);
        write_field("U" + s, u, binary);
        write_field("T" + s, t, binary);
        write_field("p" + s, pp, binary);
        write_gravity(s);
    };

    double mass0 = 0, energy0 = 0, volume0 = 0;
    /* LEVEQUE: the wind's spatial part on every node, ghosts included, with
     * the C library's sin and pow in the app's order; its time factor
     * cos(PI t / T), t = step dt, T = end_step dt, per step below */
    constexpr double PI = 3.14159265358979323846264;
    std::vector<double> scale;
    if (conv) {
        check(ctx, nsem_convection_set(ctx, U.values.data(), T.values.data()), "nsem_convection_set");
        if (leveque) {
            std::vector<double> A((size_t)M.n_all * 3);
            for (int64_t k = 0; k < M.n_all; k++) {
                const double x = M.cC[3 * k], y = M.cC[3 * k + 1];
                A[3 * k] = std::pow(std::sin(PI * x), 2.0) * std::sin(2 * PI * y);
                A[3 * k + 1] = -std::pow(std::sin(PI * y), 2.0) * std::sin(2 * PI * x);
                A[3 * k + 2] = 0.0;
            }
            check(ctx, nsem_convection_wind(ctx, A.data(), conv_order), "nsem_convection_wind");
        } else if (conv_order != 1) {
            check(ctx, nsem_convection_wind(ctx, nullptr, conv_order), "nsem_convection_wind");
        }
    } else {
        check(ctx, nsem_set_fields(ctx, rho0.data(), U.values.data(), T.values.data()), "nsem_set_fields");
        check(ctx, nsem_diagnostics(ctx, &mass0, &energy0, &volume0), "nsem_diagnostics");
    }
    if (!conv && start_step == 0) write_gravity("0");
    std::printf("--------------------------------------------\nStarting iterations.\n");
    std::fflush(stdout);

    const auto t0 = std::chrono::steady_clock::now();
    long i = start_step + 1;
    long steps = 0;
    while (i <= end_step) {
        /* advance to the next print or write point */
        long stop = std::min(end_step, i + opt.print_every - 1);
        const long next_write = ((i + write_interval - 1) / write_interval) * write_interval;
        stop = std::min(stop, next_write);
        const int chunk = (int)(stop - i + 1);
        if (conv && leveque) {
            scale.resize(chunk);
            const double period = (double)end_step * dt;
            for (int q = 0; q < chunk; q++) {
                const double time = (double)(i + q) * dt;
                scale[q] = std::cos(PI * time / period);
            }
            check(ctx, nsem_convection_step_scaled(ctx, chunk, scale.data()),
                  "nsem_convection_step_scaled");
        } else if (conv) {
            check(ctx, nsem_convection_step(ctx, chunk), "nsem_convection_step");
        } else {
            check(ctx, nsem_step(ctx, chunk, scheme, prec), "nsem_step");
        }
        steps += chunk;
        i = stop;
        std::printf("Time %f\n", (double)i * dt);
        if (!conv) {
            double mass, energy, volume;
            check(ctx, nsem_diagnostics(ctx, &mass, &energy, &volume), "nsem_diagnostics");
            std::printf("Mass loss: %.12g Energy loss %.12g Volume loss %.12g\n",
                        (mass0 - mass) / mass0, (energy0 - energy) / energy0,
                        (volume0 - volume) / volume0);
        } else {
            check(ctx, nsem_sync(ctx), "nsem_sync");
        }
        if (i % write_interval == 0) write_all(i);
        i++;
    }
    check(ctx, nsem_sync(ctx), "nsem_sync");
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    const double dof = (double)n * (conv ? 1 : 5);
    std::printf("nsem_euler: %ld steps in %.3f s, %.4g DOF-steps/s\n", steps, secs,
                steps > 0 ? dof * steps / secs : 0.0);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    const Options opt = parse_args(argc, argv);
    try {
        return run(opt);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "nsem_euler: %s\n", e.what());
        return 1;
    }
}
