/*
 * Oracle harness linked against the reference NebulaSEM library.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile.ref into oracle/_ref
 * (never shipped, never on the product path).  It drives the reference's own
 * operators -- divf/rusanov/cds/div_flux (src/field/field.h:2881-2943,
 * 3086-3117, 3417-3478), applyExplicitBCs (field.h:2586-2727) and the
 * euler-app operator chain (apps/euler/euler.cpp:104-258) -- and dumps
 * geometry, initial state, right-hand sides and SSP-RK3 trajectories as raw
 * little-endian float64 / uint32 files for the golden fixtures.
 *
 *   euler_oracle <controls> setup <outdir>   (also fld_rho/U/T: the step-0 fields)
 *   euler_oracle <controls> rk3 <outdir> <nsteps> <dump_every> [pert]
 *   euler_oracle <controls> rk3time <nsteps>
 *
 * Coupled SSP-RK3 (the reference's nonlinear Euler path has no RK3; its
 * RK branch of ddt degenerates to forward Euler, field.h:3805-3831): every
 * stage evaluates the three equations of euler.cpp:193-258 on the SAME stage
 * state, L = -Su/cV per conserved variable (rho, rho*U, rho*theta), then
 *   u1 = u0 + dt*L0
 *   u2 = 0.75*u0 + 0.25*(u1 + dt*L1)
 *   u3 = (1/3)*u0 + (2/3)*(u2 + dt*L2)
 * with each product and sum rounded separately (no FMA).
 */
#include "solve.h"
#include "iteration.h"
#include "wrapper.h"
#include "properties.h"

#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

namespace {

std::string g_out;

template <typename T>
void dump_raw(const std::string& name, const T* p, size_t n) {
    std::string path = g_out + "/" + name;
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
    fwrite(p, sizeof(T), n, f);
    fclose(f);
}

/* fields live for the whole run; pointers are set up in main */
struct Model {
    ScalarCellField* rho;
    VectorCellField* U;
    ScalarCellField* T;     /* full potential temperature during stages */
    ScalarCellField* p;
    VectorCellField* g;
    ScalarCellField* p_ref;
    ScalarCellField* rho_ref;
    ScalarCellField* gh;
    Scalar P0, R, cp, cv, gamma, T0;
    Scalar nu;              /* artificial viscosity (diffusion YES), else 0 */
};

/* Residuals Su of the three equations of the euler app (euler.cpp:181-258)
 * for the current rho, U, T(full theta) fields; ghosts refreshed here. */
void residual(Model& m, ScalarCellField& r_rho, VectorCellField& r_U,
              ScalarCellField& r_T) {
    using namespace Mesh;
    ScalarCellField& rho = *m.rho;
    VectorCellField& U = *m.U;
    ScalarCellField& T = *m.T;
    ScalarCellField& p = *m.p;
    const Scalar P0 = m.P0, R = m.R, p_gamma = m.gamma;

    applyExplicitBCs(rho, true);
    applyExplicitBCs(U, true);
    applyExplicitBCs(T, true);

    /* euler.cpp:211-213 */
    p = P0 * pow((rho * T * R) / P0, p_gamma);
    applyExplicitBCs(p, true);
    p -= *m.p_ref;

    /* euler.cpp:184-186 */
    VectorCellField Fc = flxc(rho * U);
    ScalarFacetField lambdaMax = (cds(mag(U)) + cds(sqrt(p_gamma * R * T))) / 2;
    /* euler.cpp:189-190: mu = rho viscosity with diffusion YES */
    ScalarCellField mu = Scalar(0);
    if (m.nu != 0) mu = rho * m.nu;

    /* rho equation, euler.cpp:199-203 */
    {
        VectorCellField fq = U * rho;
        ScalarFacetField Fr = flx(U);
        r_rho = divf(fq, false, &Fr, &rho, &lambdaMax);
    }
    /* U equation, euler.cpp:218-236 */
    {
        ScalarFacetField F = flx(rho * U);
        ScalarCellField Sp = Scalar(0);
        VectorCellField Sc = Vector(0.0);
        Sc += (rho - *m.rho_ref) * (*m.g);
        TensorCellField fq = mul(Fc, U) + TensorCellField(Constants::I_T) * p -
                             mu * gradf<true>(U, true);
        VectorCellField q = rho * U;
        VectorCellMatrix M = divf(fq, false, &F, &q, &lambdaMax) - src(U, Sc, Sp);
        r_U = M.Su;
    }
    /* T equation, euler.cpp:248-254 */
    {
        ScalarFacetField F = flx(rho * U);
        ScalarCellField imu = mu * (1 / Fluid::Pr);
        VectorCellField fq = Fc * T - imu * gradf<true>(T, true);
        ScalarCellField q = rho * T;
        r_T = divf(fq, false, &F, &q, &lambdaMax);
    }
}

/* conserved state on interior nodes, SoA: rho, rhou, rhov, rhow, rhotheta */
struct State {
    std::vector<Scalar> v[5];
    void resize(size_t n) { for (auto& a : v) a.assign(n, 0); }
};

void load_primitive(Model& m, const State& s) {
    ScalarCellField& rho = *m.rho;
    VectorCellField& U = *m.U;
    ScalarCellField& T = *m.T;
    for (Int i = 0; i < Mesh::gBCSfield; i++) {
        Scalar r = s.v[0][i];
        rho[i] = r;
        U[i][0] = s.v[1][i] / r;
        U[i][1] = s.v[2][i] / r;
        U[i][2] = s.v[3][i] / r;
        T[i] = s.v[4][i] / r;
    }
}

void tendency(Model& m, const State& s, State& L) {
    load_primitive(m, s);
    ScalarCellField r_rho, r_T;
    VectorCellField r_U;
    residual(m, r_rho, r_U, r_T);
    for (Int i = 0; i < Mesh::gBCSfield; i++) {
        Scalar cv = Mesh::cV[i];
        L.v[0][i] = -(r_rho[i] / cv);
        L.v[1][i] = -(r_U[i][0] / cv);
        L.v[2][i] = -(r_U[i][1] / cv);
        L.v[3][i] = -(r_U[i][2] / cv);
        L.v[4][i] = -(r_T[i] / cv);
    }
}

void rk3_step(Model& m, State& u, State& L, State& u1, Scalar dt) {
    const size_t n = u.v[0].size();
    const Scalar a2 = 0.75, b2 = 0.25, a3 = 1.0 / 3.0, b3 = 2.0 / 3.0;
    tendency(m, u, L);
    for (int c = 0; c < 5; c++)
        for (size_t i = 0; i < n; i++) {
            Scalar t = dt * L.v[c][i];
            u1.v[c][i] = u.v[c][i] + t;
        }
    tendency(m, u1, L);
    for (int c = 0; c < 5; c++)
        for (size_t i = 0; i < n; i++) {
            Scalar t = dt * L.v[c][i];
            Scalar s = u1.v[c][i] + t;
            Scalar a = a2 * u.v[c][i];
            Scalar b = b2 * s;
            u1.v[c][i] = a + b;
        }
    tendency(m, u1, L);
    for (int c = 0; c < 5; c++)
        for (size_t i = 0; i < n; i++) {
            Scalar t = dt * L.v[c][i];
            Scalar s = u1.v[c][i] + t;
            Scalar a = a3 * u.v[c][i];
            Scalar b = b3 * s;
            u.v[c][i] = a + b;
        }
}

void state_from_fields(Model& m, State& s) {
    s.resize(Mesh::gBCSfield);
    for (Int i = 0; i < Mesh::gBCSfield; i++) {
        Scalar r = (*m.rho)[i];
        s.v[0][i] = r;
        s.v[1][i] = r * (*m.U)[i][0];
        s.v[2][i] = r * (*m.U)[i][1];
        s.v[3][i] = r * (*m.U)[i][2];
        s.v[4][i] = r * (*m.T)[i];
    }
}

void dump_state(const std::string& tag, const State& s) {
    const char* nm[5] = {"rho", "rhou", "rhov", "rhow", "rhotheta"};
    for (int c = 0; c < 5; c++)
        dump_raw(tag + "_" + nm[c] + ".f64", s.v[c].data(), s.v[c].size());
}

/* Deterministic smooth velocity used to exercise the Rusanov jump and the
 * symmetry ghost states (the bubble starts at rest). */
void perturb_velocity(Model& m) {
    VectorCellField& U = *m.U;
    for (Int i = 0; i < Mesh::gBCSfield; i++) {
        const Vector& x = Mesh::cC[i];
        U[i][0] = 3.0 * sin(x[0] / 150.0 + 0.3) * cos(x[2] / 170.0);
        U[i][1] = (DG::NPY > 1) ? 2.0 * cos(x[1] / 130.0) * sin(x[0] / 190.0) : 0.0;
        U[i][2] = 2.5 * cos(x[2] / 110.0 + 0.1) * sin(x[0] / 210.0);
    }
    applyExplicitBCs(U, true);
}

void dump_geometry() {
    using namespace Mesh;
    using namespace DG;
    const Int nall = gALLfield;
    const Int nslot = gNFacets * NPF;
    Int meta[16] = {NPX, NPY, NPZ, NP, NPF, gBCS, gNCells, gBCSfield,
                    gALLfield, gNFacets, faceIndices[1][gNCells - 1], 0, 0, 0, 0, 0};
    dump_raw("meta.u32", meta, 16);
    std::vector<Scalar> buf;
    buf.resize(nall * 3);
    for (Int i = 0; i < nall; i++) for (int c = 0; c < 3; c++) buf[i * 3 + c] = cC[i][c];
    dump_raw("cC.f64", buf.data(), nall * 3);
    dump_raw("cV.f64", &cV[0], nall);
    buf.resize(nall * 9);
    for (Int i = 0; i < nall; i++) for (int c = 0; c < 9; c++) buf[i * 9 + c] = Jinv[i][c];
    dump_raw("Jinv.f64", buf.data(), nall * 9);
    dump_raw("FO.u32", &FO[0], nslot);
    dump_raw("FN.u32", &FN[0], nslot);
    buf.resize(nslot * 3);
    for (Int i = 0; i < nslot; i++) for (int c = 0; c < 3; c++) buf[i * 3 + c] = fN[i][c];
    dump_raw("fN.f64", buf.data(), nslot * 3);
    dump_raw("fI.f64", &fI[0], nslot);
    dump_raw("allFaces.u32", allFaces, faceIndices[1][gNCells - 1]);
    dump_raw("faceIdx0.u32", faceIndices[0], gNCells);
    dump_raw("faceIdx1.u32", faceIndices[1], gNCells);
    /* 1D tables per direction: x, w (NPd), psi, dpsi (NPd*NPd) */
    Int npd[3] = {NPX, NPY, NPZ};
    for (int d = 0; d < 3; d++) {
        char nm[32];
        snprintf(nm, sizeof nm, "xgl%d.f64", d);  dump_raw(nm, xgl[d], npd[d]);
        snprintf(nm, sizeof nm, "wgl%d.f64", d);  dump_raw(nm, wgl[d], npd[d]);
        snprintf(nm, sizeof nm, "psi%d.f64", d);  dump_raw(nm, psi[d], npd[d] * npd[d]);
        snprintf(nm, sizeof nm, "dpsi%d.f64", d); dump_raw(nm, dpsi[d], npd[d] * npd[d]);
    }
    /* per-slot boundary kind of U: 0 interior/unused, 1 NEUMANN, 2 SYMMETRY, 3 other */
    std::vector<Int> bcU(nslot, 0);
    Int fU = Util::hash_function("U");
    forEach(AllBConditions, b) {
        BasicBCondition* bc = AllBConditions[b];
        if (bc->fIndex != fU) continue;
        Int kind = (bc->cIndex == NEUMANN) ? 1 : (bc->cIndex == SYMMETRY) ? 2 : 3;
        for (Int j = 0; j < bc->bdry->size(); j++) {
            Int f = (*bc->bdry)[j];
            for (Int n = 0; n < NPF; n++) bcU[f * NPF + n] = kind;
        }
    }
    dump_raw("bcU.u32", bcU.data(), nslot);

    /* non-conforming (2:1) faces left by the adaptive refinement: the face,
     * which side is the coarse cell (gFMC 1: the neighbour, 2: the owner),
     * the coarse cell's face id and the halves of its face the mortar covers,
     * found as scatter_non_conforming does (field.h:2135-2248); and the 2:1
     * interpolation / projection tables psiRef, psiCor (dg.cpp:493-610) */
    std::vector<Int> mortar;
    for (Int fi = 0; fi < gNFacets; fi++) {
        const Int fm = gFMC[fi];
        if (fm < 1) continue;
        const Int cn = (fm == 1) ? gFNC[fi] : gFOC[fi];
        Cell& c = gCells[cn];
        Int fid = 0;
        forEach(c, j) {
            if (c[j] == fi) { fid = gFaceID[cn][j]; break; }
        }
        Vector cco = gFC[fi], ccn(0.0);
        Int nchildren = 0;
        forEach(c, j) {
            if (gFaceID[cn][j] == fid) { ccn += gFC[c[j]]; nchildren++; }
        }
        ccn /= Scalar(nchildren);
        Int oa, ob;
        if (fid == 0 || fid == 1) {
            const Int k = (fid == 0) ? 0 : (NPZ - 1);
            Vector v0 = cC[INDEX4(cn, 0, 0, k)], vx = cC[INDEX4(cn, NPX - 1, 0, k)],
                   vy = cC[INDEX4(cn, 0, NPY - 1, k)];
            oa = (dot(ccn - v0, vx - v0) >= dot(cco - v0, vx - v0)) ? 0 : 1;
            ob = (dot(ccn - v0, vy - v0) >= dot(cco - v0, vy - v0)) ? 0 : 1;
        } else if (fid == 2 || fid == 3) {
            const Int j = (fid == 2) ? 0 : (NPY - 1);
            Vector v0 = cC[INDEX4(cn, 0, j, 0)], vx = cC[INDEX4(cn, NPX - 1, j, 0)],
                   vz = cC[INDEX4(cn, 0, j, NPZ - 1)];
            oa = (dot(ccn - v0, vx - v0) >= dot(cco - v0, vx - v0)) ? 0 : 1;
            ob = (dot(ccn - v0, vz - v0) >= dot(cco - v0, vz - v0)) ? 0 : 1;
        } else {
            const Int i = (fid == 4) ? 0 : (NPX - 1);
            Vector v0 = cC[INDEX4(cn, i, 0, 0)], vy = cC[INDEX4(cn, i, NPY - 1, 0)],
                   vz = cC[INDEX4(cn, i, 0, NPZ - 1)];
            oa = (dot(ccn - v0, vy - v0) >= dot(cco - v0, vy - v0)) ? 0 : 1;
            ob = (dot(ccn - v0, vz - v0) >= dot(cco - v0, vz - v0)) ? 0 : 1;
        }
        mortar.push_back(fi);
        mortar.push_back(fm);
        mortar.push_back(fid);
        mortar.push_back(oa | (ob << 1));
    }
    dump_raw("mortar.u32", mortar.data(), mortar.size());
    for (int d = 0; d < 3; d++)
        for (int h = 0; h < 2; h++) {
            char nm[32];
            snprintf(nm, sizeof nm, "psiRef%d%d.f64", d, h);
            dump_raw(nm, psiRef[d * 2 + h], npd[d] * npd[d]);
            snprintf(nm, sizeof nm, "psiCor%d%d.f64", d, h);
            dump_raw(nm, psiCor[d * 2 + h], npd[d] * npd[d]);
        }
}

}  // namespace

int main(int argc, char* argv[]) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s <controls> setup|rk3|rk3time <outdir|nsteps> ...\n", argv[0]);
        return 2;
    }
    std::string mode = argv[2];
    MP mp(argc, argv);
    Solver::Initialize(argc, argv);
    std::istream& input = Solver::input;
    if (mode != "rk3time") g_out = argv[3];

    Int buoyancy = 1, diffusion = 1;
    {
        Util::ParamList params("general");
        Fluid::enroll(params);
        params.read(input);
    }
    {
        Scalar ur = 0;
        Util::ParamList params("euler");
        params.enroll("velocity_UR", &ur);
        params.enroll("pressure_UR", &ur);
        params.enroll("t_UR", &ur);
        params.enroll("buoyancy", new Util::BoolOption(&buoyancy));
        params.enroll("diffusion", new Util::BoolOption(&diffusion));
        Util::read_params(input, MP::printOn);
    }

    Mesh::LoadMesh(0);
    ScalarCellField p("p", READWRITE);
    VectorCellField U("U", READWRITE);
    ScalarCellField T("T", READWRITE);
    ScalarCellField rho("rho", READWRITE);
    VectorCellField g(false);
    Iteration it(0);

    using namespace Fluid;
    Model m;
    m.P0 = P0; m.cp = cp; m.cv = cv; m.T0 = T0;
    m.R = cp - cv;
    m.gamma = cp / cv;
    m.nu = diffusion ? Fluid::viscosity : 0;
    const Scalar R = m.R, p_gamma = m.gamma;

    /* hydrostatic reference state, euler.cpp:106-123 */
    ScalarCellField p_ref, rho_ref, gh;
    g.construct("gravity", WRITE);
    g = Controls::gravity;
    gh = dot(g, Mesh::cC);
    Mesh::fixedBCs<Vector>(U, g);
    applyExplicitBCs(g, true);
    p_ref = P0 * pow(1.0 + gh / (cp * T0), cp / R);
    rho_ref = (P0 / (R * T0)) * pow(p_ref / P0, 1 / p_gamma);

    /* rho from p at start, euler.cpp:136-149 */
    p += p_ref;
    Mesh::scaleBCs<Scalar>(p, p_ref, 1.0);
    applyExplicitBCs(p_ref, true);
    applyExplicitBCs(p, true);
    rho = (P0 / (R * (T + T0))) * pow(p / P0, 1 / p_gamma);
    applyExplicitBCs(rho, true);
    Mesh::scaleBCs<Scalar>(rho, rho_ref, 1);
    applyExplicitBCs(rho_ref, true);
    p -= p_ref;

    m.rho = &rho; m.U = &U; m.T = &T; m.p = &p; m.g = &g;
    m.p_ref = &p_ref; m.rho_ref = &rho_ref; m.gh = &gh;

    /* the solver's own fields at step 0 (rho, U, T = theta'), as the euler
     * app holds them when its time loop starts */
    if (mode == "setup") {
        dump_raw("fld_rho.f64", &rho[0], Mesh::gBCSfield);
        dump_raw("fld_U.f64", &U[0][0], 3 * (size_t)Mesh::gBCSfield);
        dump_raw("fld_T.f64", &T[0], Mesh::gBCSfield);
    }

    /* T holds theta' in the reference's files; stages use full theta */
    T += T0;

    if (mode == "setup") {
        dump_geometry();
        const Int nall = Mesh::gALLfield;
        dump_raw("p_ref.f64", &p_ref[0], nall);
        dump_raw("rho_ref.f64", &rho_ref[0], nall);
        dump_raw("gh.f64", &gh[0], nall);
        State s, L;
        state_from_fields(m, s);
        L.resize(Mesh::gBCSfield);
        dump_state("u0", s);
        tendency(m, s, L);
        dump_state("L0", L);
        dump_raw("p0prime.f64", &p[0], nall);
        /* perturbed velocity state */
        perturb_velocity(m);
        State sp;
        state_from_fields(m, sp);
        dump_state("up", sp);
        tendency(m, sp, L);
        dump_state("Lp", L);
        dump_raw("ppprime.f64", &p[0], nall);
        printf("setup done: %u interior nodes\n", Mesh::gBCSfield);
        return 0;
    }
    if (mode == "rk3" || mode == "rk3time") {
        Int nsteps = atoi(argv[mode == "rk3" ? 4 : 3]);
        Int every = (mode == "rk3") ? atoi(argv[5]) : 0;
        bool pert = (mode == "rk3" && argc > 6 && std::string(argv[6]) == "pert");
        if (pert) perturb_velocity(m);
        State u, L, u1;
        state_from_fields(m, u);
        L.resize(Mesh::gBCSfield);
        u1.resize(Mesh::gBCSfield);
        auto t0 = std::chrono::steady_clock::now();
        for (Int s = 1; s <= nsteps; s++) {
            rk3_step(m, u, L, u1, Controls::dt);
            if (every && (s % every == 0)) {
                char tag[32];
                snprintf(tag, sizeof tag, "s%05u", s);
                dump_state(tag, u);
            }
        }
        auto t1 = std::chrono::steady_clock::now();
        double sec = std::chrono::duration<double>(t1 - t0).count();
        printf("rk3 %u steps %.3f s  %.3f ms/stage  %.4g DOF-stages/s\n", nsteps, sec,
               1e3 * sec / (3.0 * nsteps), 5.0 * Mesh::gBCSfield * 3.0 * nsteps / sec);
        return 0;
    }
    fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
