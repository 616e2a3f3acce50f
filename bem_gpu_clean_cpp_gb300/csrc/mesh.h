// Host-side mesh object behind bem_mesh_t (the reference's class mesh,
// mesh.h:216-259).
#pragma once

#include <vector>

#include "bem_common.h"

struct bem_mesh_s {
    std::vector<double> pnts;    // 3 * N node coordinates
    std::vector<int> elems;      // 3 * E zero-based node indices
    std::vector<double> bc;      // 6 * E: ca, cb, cc as (re, im)
    std::vector<double> chief;   // 3 * M CHIEF points
    float bb[6] = {0, 0, 0, 0, 0, 0};  // xl, xu, yl, yu, zl, zu
    bool has_bb = false;

    int num_pnts() const { return (int)(pnts.size() / 3); }
    int num_elems() const { return (int)(elems.size() / 3); }
    int num_chief() const { return (int)(chief.size() / 3); }
    void default_bc();
    void validate() const;
};

namespace bem {

void read_obj_reference(bem_mesh_s &m, const char *path);
void read_obj_robust(bem_mesh_s &m, const char *path);
void read_ply(bem_mesh_s &m, const char *path);

struct MeshOrientReport {
    int flipped, components, open_edges, nonmanifold;
    double volume;   // enclosed volume of the closed components after orientation
};
MeshOrientReport orient_mesh(bem_mesh_s &m);
void make_icosphere(bem_mesh_s &m, int subdiv, double radius);
void make_geodesic(bem_mesh_s &m, int nu, double radius);
void map_perturbed_ellipsoid(bem_mesh_s &m, double a, double b, double c, int lmax, double amp,
                             unsigned long long seed);
void fibonacci_sphere(int n, double radius, double *out);
void find_bb(bem_mesh_s &m, float threshold);
void gen_chief(bem_mesh_s &m, int num, float threshold);

// GPU test of CHIEF candidates (chief.cu): for each candidate point/direction
// returns 1 when it is accepted (odd ray crossings and min node distance >=
// threshold), else 0.
void chief_test_candidates(const std::vector<float> &pnts_f, const std::vector<int> &elems,
                           const std::vector<float> &cand_pts, const std::vector<float> &cand_dirs,
                           float threshold, std::vector<int> &accepted);

}  // namespace bem
