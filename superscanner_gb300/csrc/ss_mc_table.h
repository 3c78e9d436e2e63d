// ss_mc_table.h — the marching-cubes case table, generated at compile time.
//
// Cube conventions of the classic marching cubes that Open3D's
// ScalableTSDFVolume::ExtractTriangleMesh runs on the volume units the
// reference hands it (GPUVoxelGrid.cpp:200-251): corners
//   0 (0,0,0) 1 (1,0,0) 2 (1,1,0) 3 (0,1,0) 4 (0,0,1) 5 (1,0,1) 6 (1,1,1) 7 (0,1,1),
// edges 0-3 around the z = 0 face (0-1, 1-2, 2-3, 3-0), 4-7 around the z = 1
// face (4-5, 5-6, 6-7, 7-4), 8-11 upwards (0-4, 1-5, 2-6, 3-7); bit i of the
// case index is set when corner i's sdf is negative. The triangles of each
// case are derived here instead of read from a published table: on each cube
// face the sign-changing edges are paired into segments (two crossings: one
// segment; four, corners alternating: each negative corner is cut off on its
// own, a rule that depends on the face's corners only, so the two cubes
// sharing a face agree and the surface is closed), the segments are chained
// into closed loops, each loop is oriented so that its normal (edge
// midpoints, Newell's method) points from the negative to the positive
// corners, and fanned into triangles from its first vertex. The vertices are
// those of marching cubes (one per sign-changing edge); the polygons equal
// the published table's except on faces with four crossings, and a polygon of
// more than three vertices may be split along other diagonals.
#pragma once

namespace ss {

constexpr int kMcMaxTris = 6;

struct McTable {
    signed char tri[256][kMcMaxTris * 3 + 1];  // edge triples, -1 terminated
    unsigned short edges[256];                 // sign-changing edges of the case (bit per edge)
};

namespace mc_detail {

constexpr int kEdgeCorner[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                    {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
constexpr int kCornerPos[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
// faces: 4 corners in cyclic order and the 4 edges between consecutive corners
constexpr int kFaceCorner[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};
constexpr int kFaceEdge[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 9, 4, 8}, {2, 10, 6, 11}, {3, 11, 7, 8}, {1, 10, 5, 9}};

constexpr McTable make() {
    McTable t{};
    for (int cs = 0; cs < 256; cs++) {
        for (int k = 0; k < kMcMaxTris * 3 + 1; k++) t.tri[cs][k] = -1;
        unsigned short em = 0;
        for (int e = 0; e < 12; e++) {
            const bool a = (cs >> kEdgeCorner[e][0]) & 1, b = (cs >> kEdgeCorner[e][1]) & 1;
            if (a != b) em |= (unsigned short)(1u << e);
        }
        t.edges[cs] = em;
        // each crossing edge has two neighbours, one through each of its two faces
        int nb[12][2] = {};
        int nn[12] = {};
        for (int f = 0; f < 6; f++) {
            int cr[4] = {}, nc = 0;
            for (int q = 0; q < 4; q++)
                if (em & (1u << kFaceEdge[f][q])) cr[nc++] = q;
            if (nc == 2) {
                const int e0 = kFaceEdge[f][cr[0]], e1 = kFaceEdge[f][cr[1]];
                nb[e0][nn[e0]++] = e1;
                nb[e1][nn[e1]++] = e0;
            } else if (nc == 4) {
                // corners alternate: cut off each negative corner (its two face edges)
                for (int q = 0; q < 4; q++) {
                    const int corner = kFaceCorner[f][q];
                    if (!((cs >> corner) & 1)) continue;
                    const int ea = kFaceEdge[f][q], eb = kFaceEdge[f][(q + 3) % 4];  // edges at corner q
                    nb[ea][nn[ea]++] = eb;
                    nb[eb][nn[eb]++] = ea;
                }
            }
        }
        // chain into loops, fan each
        bool used[12] = {};
        int out = 0;
        for (int e = 0; e < 12; e++) {
            if (!(em & (1u << e)) || used[e]) continue;
            int loop[12] = {}, n = 0;
            int prev = -1, cur = e;
            while (!used[cur]) {
                used[cur] = true;
                loop[n++] = cur;
                const int nx = nb[cur][0] != prev ? nb[cur][0] : nb[cur][1];
                prev = cur;
                cur = nx;
            }
            // Newell normal of the loop through the edge midpoints (doubled coordinates)
            int nxs = 0, nys = 0, nzs = 0, dx = 0, dy = 0, dz = 0;
            for (int k = 0; k < n; k++) {
                const int ea = loop[k], eb = loop[(k + 1) % n];
                int pa[3] = {}, pb[3] = {};
                for (int c = 0; c < 3; c++) {
                    pa[c] = kCornerPos[kEdgeCorner[ea][0]][c] + kCornerPos[kEdgeCorner[ea][1]][c];
                    pb[c] = kCornerPos[kEdgeCorner[eb][0]][c] + kCornerPos[kEdgeCorner[eb][1]][c];
                }
                nxs += (pa[1] - pb[1]) * (pa[2] + pb[2]);
                nys += (pa[2] - pb[2]) * (pa[0] + pb[0]);
                nzs += (pa[0] - pb[0]) * (pa[1] + pb[1]);
                // negative -> positive corner of this crossing edge
                const int c0 = kEdgeCorner[ea][0], c1 = kEdgeCorner[ea][1];
                const int neg = ((cs >> c0) & 1) ? c0 : c1, pos = neg == c0 ? c1 : c0;
                dx += kCornerPos[pos][0] - kCornerPos[neg][0];
                dy += kCornerPos[pos][1] - kCornerPos[neg][1];
                dz += kCornerPos[pos][2] - kCornerPos[neg][2];
            }
            const bool flip = nxs * dx + nys * dy + nzs * dz < 0;
            for (int k = 1; k + 1 < n; k++) {
                const int a = loop[0], b = loop[k], c = loop[k + 1];
                t.tri[cs][out++] = (signed char)a;
                t.tri[cs][out++] = (signed char)(flip ? c : b);
                t.tri[cs][out++] = (signed char)(flip ? b : c);
            }
        }
    }
    return t;
}

}  // namespace mc_detail

constexpr McTable kMcTable = mc_detail::make();

}  // namespace ss
