/*
 * Mesh of a case directory for the host driver.
 *
 * Input: the block description the reference's mesh app reads
 * (apps/mesh/meshApp.cpp:70-230: key points, hex blocks `8{...} <grading>
 * 3{nx ny nz} ...`, named boundary patches `name 4{a b c d}...`, `default
 * name`).  Supported: one hexahedral block with straight edges forming a
 * parallelepiped (axis-aligned, or rotated / sheared as the reference's
 * srtb-inclined example), uniform spacing (`linear`, or `wall`/`geometric`
 * with all factors 1); a `delete` patch on the two faces of the block's second
 * axis, one element thick, makes the case two-dimensional (npy 0).  Anything
 * else (curved edges, several blocks, grading) is rejected with a message:
 * the driver has no CPU path to fall back to.
 *
 * Metric of a non-axis-aligned block: the reference's pseudo-inverse
 * (dg.cpp:412-476) Jinv = ((J^T J)^-1 J^T)^T of the constant element Jacobian
 * J = [e_0/2, e_1/2, e_2/2] (a collapsed direction's column and inverse
 * diagonal zero), node weights V_e w_i w_j w_k / 8, face area vectors e_b x e_c.
 *
 * Output: the arrays of the reference's Mesh:: / DG:: layout for that box
 * (the nsem_mesh_desc of the C ABI), built with the reference's conventions:
 * LGL nodes and Lagrange tables as src/field/dg.cpp:32-143, face slots and
 * weights as DG::init_geom (dg.cpp:323-410), node weights cV = V w_i w_j w_k
 * / 8, metric Jinv = diag(2/h).  Node coordinates are the exact affine
 * values; element, face and ghost-cell numbering are canonical (element z
 * fastest, then y, then x; interior faces z, y, x; boundary faces z-, z+,
 * y-, y+, x-, x+), so the discretisation is the reference's up to the order
 * of the face sums and the last bits of the geometry.
 */
#ifndef NSEM_DRIVER_CASE_MESH_H
#define NSEM_DRIVER_CASE_MESH_H

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "nsem.h"

namespace nsem_driver {

/* one side of the box: axis 0/1/2 (x/y/z), sign -1/+1 */
struct BoxSide {
    int axis, sign;
};

struct BlockDesc {
    std::array<double, 3> lo{}, hi{};      /* box extent (axis-aligned blocks) */
    std::array<int, 3> n{};                /* elements per axis: global x, y, z for an
                                              axis-aligned block, else the block's own
                                              axes v0->v1, v0->v3, v0->v4 */
    /* patch name of each side, in the order z-, z+, y-, y+, x-, x+ of those axes
     * ("" if deleted) */
    std::array<std::string, 6> patch;
    bool two_d = false;                    /* y faces deleted, one element in y */
    /* a block whose edges are not along the coordinate axes (rotated or
     * sheared parallelepiped): x = origin + sum_a xi_a E[a], xi_a in [0, 1] */
    bool affine = false;
    std::array<double, 3> origin{};
    std::array<std::array<double, 3>, 3> E{};
};

/* parse the block description file; throws std::runtime_error */
BlockDesc read_block_description(const std::string& path);

struct CaseMesh {
    int npx = 0, npy = 0, npz = 0, np = 0, npf = 0;
    int64_t n_elem = 0, n_cells = 0, n_face = 0, n_int = 0, n_all = 0;
    std::vector<double> cC, cV, Jinv, fN, fI;
    std::vector<uint32_t> FO, FN, all_faces, face_idx0, face_idx1, bc_U;
    std::array<std::vector<double>, 3> xgl, wgl, psi, dpsi;
    /* patch index (into BlockDesc::patch) of every boundary face slot, -1 inside */
    std::vector<int8_t> slot_side;
    nsem_mesh_desc desc() const;
};

/* LGL nodes and weights on [-1, 1] (dg.cpp:32-101) */
void lgl(int n, std::vector<double>& x, std::vector<double>& w);
/* psi[j*n+s] = l_j(x_s), dpsi[s*n+i] = l_i'(x_s) (dg.cpp:103-143) */
void lagrange_tables(const std::vector<double>& x, std::vector<double>& psi,
                     std::vector<double>& dpsi);

/* DG mesh of the block for LGL points per direction (npx, npy, npz);
 * side_bc[s] is the velocity condition of side s (1 NEUMANN, 2 SYMMETRY) */
CaseMesh build_box_mesh(const BlockDesc& b, int npx, int npy, int npz,
                        const std::array<uint32_t, 6>& side_bc);

}  // namespace nsem_driver

#endif
