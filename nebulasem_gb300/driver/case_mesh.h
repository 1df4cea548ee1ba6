/*
 * Mesh of a case directory for the host driver.
 *
 * Input: the block description the reference's mesh app reads
 * (apps/mesh/meshApp.cpp:70-230: key points, hex blocks `8{...} <grading>
 * 3{nx ny nz} ... [edges n{...}]`, named boundary patches `name 4{a b c
 * d}...`, `default name`).  Supported: one hexahedral block, either with
 * straight edges forming a parallelepiped (axis-aligned, or rotated / sheared
 * as the reference's srtb-inclined example) or with curved edges (any 8
 * corners); `linear`, `geometric` or `wall` spacing with grading factors
 * (hexMesh.cpp:48-100); a `delete` patch on the two faces of the block's
 * second axis, one element thick, makes the case two-dimensional (npy 0).
 * Anything else (several blocks, mixed spacing types) is rejected with a
 * message: the driver has no CPU path to fall back to.
 *
 * Geometry, for every block, as the reference's mesh app and LoadMesh form
 * it, operation by operation so that the arrays agree to the bit: the
 * block's vertex lattice by transfinite interpolation of its corners, edges
 * (straight, arcs through the key point, or the bump shapes of
 * hexMesh.cpp:20-45) and faces; each element straight-edged between its 8
 * vertices (dg.cpp:167-300), its nodes by transfinite interpolation, the
 * metric per node from the LGL derivative of the node coordinates and the
 * pseudo-inverse ((J^T J)^-1 J^T)^T with a collapsed direction's diagonal
 * zero (dg.cpp:412-476); the node weights from the element volume and the
 * face weights from the face area vectors as Mesh::calcGeometry forms them
 * (mesh.cpp:450-520: triangle fans about the vertex centroid, pyramids about
 * the cell centre).
 *
 * Output: the arrays of the reference's Mesh:: / DG:: layout for that box
 * (the nsem_mesh_desc of the C ABI), built with the reference's conventions:
 * LGL nodes and Lagrange tables as src/field/dg.cpp:32-143, face slots and
 * weights as DG::init_geom (dg.cpp:323-410).  Element, face and ghost-cell
 * numbering are canonical (element k fastest, then j, then i; interior faces
 * normal to k, j, i; boundary faces k-, k+, j-, j+, i-, i+); each node's
 * face terms are summed in the cell's face order k-, k+, j-, j+, i-, i+ as in
 * the reference, so its examples run bit-identically.
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
    std::array<int, 3> n{};                /* elements along the block's own axes
                                              v0->v1, v0->v3, v0->v4 (i, j, k) */
    /* patch name of each side, in the order k-, k+, j-, j+, i-, i+ of those axes
     * ("" if deleted) */
    std::array<std::string, 6> patch;
    /* 2D case: the axis (1 = j, 2 = k) whose two faces are deleted, one
     * element thick along it (the mesh app's `delete` patch); -1 in 3D */
    int del_axis = -1;
    /* the 8 corners in hex order and the 12 edges; curved edges from
     * `edges n{ arc|cosine|gaussian|ridge|schar side key [scale] }` */
    bool curved = false;
    bool wall = false;                     /* `wall` spacing: mirrored edge parameters */
    std::array<double, 12> factor{};       /* grading factor per edge (geometric / wall) */
    std::array<std::array<double, 3>, 8> corner{};
    struct Edge {
        int type = 0;                      /* 0 straight, 1 arc, 2 cosine, 3 gaussian, 4 ridge, 5 schar */
        std::array<double, 3> key{};       /* the edge's third key point */
        double scale = 1.0;
    };
    std::array<Edge, 12> edge{};
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
