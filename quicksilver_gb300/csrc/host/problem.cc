// Host-side construction of the read-only problem tables from a deck.
//
// This is set-up work the reference does once in initMC (initMC.cc:53-320);
// it is restated here with the same floating-point expressions so that every
// table is bitwise equal to the reference's:
//   * energy group edges           NuclearData.cc:105-119
//   * reaction cross sections      NuclearData.cc:12-42, 121-187
//   * material isotope lists       initMC.cc:130-197 (materials in name order)
//   * FCC-hex mesh nodes           GlobalFccGrid.cc:17-131
//   * 24 facets per cell           MC_Domain.cc:41-50, 196-317
//   * facet planes                 MC_Facet_Geometry.hh:18-39
//   * cell volume / material / id  MC_Domain.cc:320-394, 403-450
// The whole grid is one domain (cell index = global cell id, x fastest), which
// is what the reference builds for xDom=yDom=zDom=1 on one rank
// (initMC.cc:240-320, MeshPartition.cc:127-170).
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "deck.h"
#include "status.h"

namespace qsg {

// Cell-local point numbers of the 24 triangular facets: 6 faces x 4
// triangles, each triangle = two hex corners + the face centre.  The table is
// fixed by the reference's mesh convention (MC_Domain.cc:41-46) and must match
// it so that facet numbering, tie-breaks and adjacency agree.
static const int32_t kFacetLocalPoints[24][3] = {
    {1, 3, 8}, {3, 7, 8}, {7, 5, 8}, {5, 1, 8},  {0, 4, 9},  {4, 6, 9},  {6, 2, 9},  {2, 0, 9},
    {3, 2, 10}, {2, 6, 10}, {6, 7, 10}, {7, 3, 10}, {0, 1, 11}, {1, 5, 11}, {5, 4, 11}, {4, 0, 11},
    {4, 5, 12}, {5, 7, 12}, {7, 6, 12}, {6, 4, 12}, {0, 2, 13}, {2, 3, 13}, {3, 1, 13}, {1, 0, 13}};

// Facet on the neighbouring cell that shares a triangle (MC_Domain.cc:48-50).
static const int32_t kOpposingFacet[24] = {7, 6, 5, 4, 3, 2, 1, 0, 12, 15, 14, 13,
                                           8, 11, 10, 9, 20, 23, 22, 21, 16, 19, 18, 17};

// Node-lattice offsets (x, y, z, basis) of a cell's 14 points
// (GlobalFccGrid.cc:48-70): 8 corners then 6 face centres.
static const int32_t kCornerOffset[14][4] = {
    {0, 0, 0, 0}, {1, 0, 0, 0}, {0, 1, 0, 0}, {1, 1, 0, 0}, {0, 0, 1, 0}, {1, 0, 1, 0}, {0, 1, 1, 0},
    {1, 1, 1, 0}, {1, 0, 0, 1}, {0, 0, 0, 1}, {0, 1, 0, 2}, {0, 0, 0, 2}, {0, 0, 1, 3}, {0, 0, 0, 3}};

// Face neighbour offsets, +x -x +y -y +z -z (GlobalFccGrid.cc:142-158).
static const int32_t kFaceOffset[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};

struct Vec3 {
    double x, y, z;
};

}  // namespace qsg

struct QsgHostProblem {
    int32_t num_groups = 0;
    std::vector<double> energies;
    std::vector<int32_t> isotope_reaction_offset;
    std::vector<int32_t> reaction_type;
    std::vector<double> reaction_nubar;
    std::vector<double> reaction_xs;
    std::vector<int32_t> material_isotope_offset;
    std::vector<int32_t> material_isotope_gid;
    std::vector<double> material_atom_fraction;
    std::vector<double> material_mass;
    std::vector<double> material_source_rate;
    std::vector<std::string> material_names;
    int32_t num_cells = 0;
    std::vector<double> nodes;
    std::vector<int32_t> cell_points;
    std::vector<int32_t> facet_local_points;
    std::vector<double> facet_planes;
    std::vector<int32_t> facet_event;
    std::vector<int32_t> facet_adjacent_cell;
    std::vector<int32_t> facet_adjacent_facet;
    std::vector<int32_t> cell_material;
    std::vector<double> cell_number_density;
    std::vector<double> cell_volume;
    std::vector<uint64_t> cell_id;
    double time_step = 0.0;
};

namespace qsg {
namespace {

// Polynomial::operator(), NuclearData.hh:13-27.
double poly_eval(const CrossSectionSpec& p, double xx)
{
    return p.ee + xx * (p.dd + xx * (p.cc + xx * (p.bb + xx * (p.aa))));
}

// NuclearData::NuclearData, NuclearData.cc:105-119.
std::vector<double> energy_edges(int G, double e_low, double e_high)
{
    if (!(e_low < e_high)) throw std::runtime_error("deck: eMin must be below eMax");
    if (G < 1) throw std::runtime_error("deck: nGroups must be positive");
    std::vector<double> e(G + 1);
    e[0] = e_low;
    e[G] = e_high;
    double log_low = log(e_low);
    double log_high = log(e_high);
    double delta = (log_high - log_low) / (G + 1.0);
    for (int i = 1; i < G; i++) {
        double log_value = log_low + delta * i;
        e[i] = exp(log_value);
    }
    return e;
}

// NuclearDataReaction ctor, NuclearData.cc:12-42.
void reaction_table(const std::vector<double>& e, const CrossSectionSpec& poly, double reaction_xs, double* out)
{
    const int G = (int)e.size() - 1;
    for (int g = 0; g < G; g++) {
        double energy = (e[g] + e[g + 1]) / 2.0;
        out[g] = pow(10.0, poly_eval(poly, log10(energy)));
    }
    double normalization = 0.0;
    for (int g = 0; g < G; g++)
        if (e[g + 1] >= 1.) {
            normalization = out[g];
            break;
        }
    if (!(normalization > 0.)) throw std::runtime_error("deck: cross-section normalisation at 1 MeV is not positive");
    double scale = reaction_xs / normalization;
    for (int g = 0; g < G; g++) out[g] *= scale;
}

const CrossSectionSpec& find_xs(const Deck& d, const std::string& name, const std::string& mat)
{
    auto it = d.cross_sections.find(name);
    if (it == d.cross_sections.end())
        throw std::runtime_error("deck: material '" + mat + "' names unknown CrossSection '" + name + "'");
    return it->second;
}

// NuclearData::addIsotope, NuclearData.cc:121-187.
void add_isotope(QsgHostProblem& hp, const Deck& d, const MaterialSpec& mp)
{
    const int G = hp.num_groups;
    const CrossSectionSpec& fission = find_xs(d, mp.fission_cross_section, mp.name);
    const CrossSectionSpec& scatter = find_xs(d, mp.scattering_cross_section, mp.name);
    const CrossSectionSpec& absorb = find_xs(d, mp.absorption_cross_section, mp.name);
    double nu_bar = fission.nu_bar;  // initMC.cc:175
    double total_weight = mp.fission_ratio + mp.scattering_ratio + mp.absorption_ratio;
    int nr = mp.n_reactions;
    int n_fission = nr / 3, n_scatter = nr / 3, n_absorb = nr / 3;
    switch (nr % 3) {
    case 1: ++n_scatter; break;
    case 2: ++n_scatter; ++n_fission; break;
    default: break;
    }
    double fission_xs = (mp.total_cross_section * mp.fission_ratio) / (n_fission * total_weight);
    double scatter_xs = (mp.total_cross_section * mp.scattering_ratio) / (n_scatter * total_weight);
    double absorb_xs = (mp.total_cross_section * mp.absorption_ratio) / (n_absorb * total_weight);
    for (int r = 0; r < nr; r++) {
        int type;
        const CrossSectionSpec* poly;
        double xs;
        switch (r % 3) {
        case 0: type = QSG_REACT_SCATTER; poly = &scatter; xs = scatter_xs; break;
        case 1: type = QSG_REACT_FISSION; poly = &fission; xs = fission_xs; break;
        default: type = QSG_REACT_ABSORPTION; poly = &absorb; xs = absorb_xs; break;
        }
        hp.reaction_type.push_back(type);
        hp.reaction_nubar.push_back(nu_bar);
        size_t off = hp.reaction_xs.size();
        hp.reaction_xs.resize(off + G);
        reaction_table(hp.energies, *poly, xs, &hp.reaction_xs[off]);
    }
    hp.isotope_reaction_offset.push_back((int32_t)hp.reaction_type.size());
}

// isInside, MC_Domain.cc:407-432.
bool is_inside(const GeometrySpec& g, const Vec3& r)
{
    if (g.shape == GeometrySpec::BRICK)
        return (r.x >= g.x_min && r.x <= g.x_max) && (r.y >= g.y_min && r.y <= g.y_max) &&
               (r.z >= g.z_min && r.z <= g.z_max);
    double dx = r.x - g.x_center, dy = r.y - g.y_center, dz = r.z - g.z_center;
    return sqrt(dx * dx + dy * dy + dz * dz) <= g.radius;
}

}  // namespace

static void build_problem(const Deck& d, QsgHostProblem& hp)
{
    const SimulationSpec& s = d.sim;
    if (s.nx < 1 || s.ny < 1 || s.nz < 1) throw std::runtime_error("deck: nx, ny, nz must be positive");
    int bc = boundary_condition_code(s.boundary_condition);
    if (bc < 0) throw std::runtime_error("deck: boundaryCondition must be reflect, escape or octant");
    if ((int64_t)s.nx * s.ny * s.nz > (int64_t)INT32_MAX / 24)
        throw std::runtime_error("deck: mesh too large for 32-bit facet indexing");

    // ---- nuclear data and materials (initMC.cc:130-197) ----
    hp.num_groups = s.n_groups;
    hp.energies = energy_edges(s.n_groups, s.e_min, s.e_max);
    hp.isotope_reaction_offset.assign(1, 0);
    hp.material_isotope_offset.assign(1, 0);
    for (const auto& kv : d.materials) {
        const MaterialSpec& mp = kv.second;
        if (mp.n_isotopes < 1 || mp.n_reactions < 1)
            throw std::runtime_error("deck: material '" + mp.name + "' needs nIsotopes, nReactions >= 1");
        for (int i = 0; i < mp.n_isotopes; i++) {
            int gid = (int)hp.isotope_reaction_offset.size() - 1;
            add_isotope(hp, d, mp);
            hp.material_isotope_gid.push_back(gid);
            hp.material_atom_fraction.push_back(1.0 / mp.n_isotopes);  // initMC.cc:193
        }
        hp.material_isotope_offset.push_back((int32_t)hp.material_isotope_gid.size());
        hp.material_mass.push_back(mp.mass);
        hp.material_source_rate.push_back(mp.source_rate);
        hp.material_names.push_back(mp.name);
    }

    // ---- mesh (GlobalFccGrid + MC_Mesh_Domain + MC_Domain) ----
    const int nx = s.nx, ny = s.ny, nz = s.nz;
    const double dx = s.lx / nx, dy = s.ly / ny, dz = s.lz / nz;  // GlobalFccGrid.cc:26-28
    const int64_t NX = nx + 1, NY = ny + 1, NZ = nz + 1;
    const int64_t num_nodes = NX * NY * NZ * 4;
    hp.nodes.resize(num_nodes * 3);
    for (int64_t idx = 0; idx < num_nodes; idx++) {
        // IndexToTuple4 (IndexToTuple4.hh) then GlobalFccGrid::nodeCoord (GlobalFccGrid.cc:112-131)
        int64_t t = idx;
        int tx = (int)(t % NX); t /= NX;
        int ty = (int)(t % NY); t /= NY;
        int tz = (int)(t % NZ);
        int tb = (int)(t / NZ);
        double bx = 0., by = 0., bz = 0.;
        if (tb == 1) { by = dy / 2.0; bz = dz / 2.0; }
        if (tb == 2) { bx = dx / 2.0; bz = dz / 2.0; }
        if (tb == 3) { bx = dx / 2.0; by = dy / 2.0; }
        double rx = tx * dx, ry = ty * dy, rz = tz * dz;
        hp.nodes[idx * 3 + 0] = rx + bx;
        hp.nodes[idx * 3 + 1] = ry + by;
        hp.nodes[idx * 3 + 2] = rz + bz;
    }

    const int64_t C = (int64_t)nx * ny * nz;
    hp.num_cells = (int32_t)C;
    hp.cell_points.resize(C * 14);
    hp.facet_local_points.assign(&kFacetLocalPoints[0][0], &kFacetLocalPoints[0][0] + 72);
    hp.facet_planes.resize(C * 96);
    hp.facet_event.resize(C * 24);
    hp.facet_adjacent_cell.resize(C * 24);
    hp.facet_adjacent_facet.resize(C * 24);
    hp.cell_material.resize(C);
    hp.cell_number_density.assign(C, 1.0);  // MC_Domain.cc:387
    hp.cell_volume.resize(C);
    hp.cell_id.resize(C);

    // boundary events per face, getBoundaryCondition (MC_Domain.cc:455-471)
    int face_bc[6];
    for (int f = 0; f < 6; f++) {
        if (bc == 0) face_bc[f] = QSG_ADJ_BOUNDARY_REFLECTION;
        else if (bc == 1) face_bc[f] = QSG_ADJ_BOUNDARY_ESCAPE;
        else face_bc[f] = (f % 2 == 0) ? QSG_ADJ_BOUNDARY_ESCAPE : QSG_ADJ_BOUNDARY_REFLECTION;
    }

    for (int64_t c = 0; c < C; c++) {
        int ix = (int)(c % nx), iy = (int)((c / nx) % ny), iz = (int)(c / ((int64_t)nx * ny));
        int32_t* pts = &hp.cell_points[c * 14];
        for (int p = 0; p < 14; p++) {
            int64_t tx = ix + kCornerOffset[p][0], ty = iy + kCornerOffset[p][1], tz = iz + kCornerOffset[p][2];
            int64_t tb = kCornerOffset[p][3];
            pts[p] = (int32_t)(tx + NX * (ty + NY * (tz + NZ * tb)));  // Tuple4ToIndex.hh
        }
        auto node = [&](int local) {
            const double* v = &hp.nodes[(int64_t)pts[local] * 3];
            return Vec3{v[0], v[1], v[2]};
        };
        // facet planes, MC_General_Plane(r0, r1, r2), MC_Facet_Geometry.hh:18-39
        for (int f = 0; f < 24; f++) {
            Vec3 r0 = node(kFacetLocalPoints[f][0]), r1 = node(kFacetLocalPoints[f][1]),
                 r2 = node(kFacetLocalPoints[f][2]);
            double A = ((r1.y - r0.y) * (r2.z - r0.z)) - ((r1.z - r0.z) * (r2.y - r0.y));
            double B = ((r1.z - r0.z) * (r2.x - r0.x)) - ((r1.x - r0.x) * (r2.z - r0.z));
            double Cc = ((r1.x - r0.x) * (r2.y - r0.y)) - ((r1.y - r0.y) * (r2.x - r0.x));
            double D = -1.0 * (A * r0.x + B * r0.y + Cc * r0.z);
            double magnitude = sqrt(A * A + B * B + Cc * Cc);
            if (magnitude == 0.0) {
                A = 1.0;
                magnitude = 1.0;
            }
            double inv = 1.0 / magnitude;
            A *= inv;
            B *= inv;
            Cc *= inv;
            D *= inv;
            double* pl = &hp.facet_planes[(c * 24 + f) * 4];
            pl[0] = A; pl[1] = B; pl[2] = Cc; pl[3] = D;
        }
        // face neighbours and facet adjacency (GlobalFccGrid.cc:88-104, MC_Domain.cc:253-317)
        for (int face = 0; face < 6; face++) {
            int jx = ix + kFaceOffset[face][0], jy = iy + kFaceOffset[face][1], jz = iz + kFaceOffset[face][2];
            jx = jx < 0 ? 0 : (jx > nx - 1 ? nx - 1 : jx);
            jy = jy < 0 ? 0 : (jy > ny - 1 ? ny - 1 : jy);
            jz = jz < 0 ? 0 : (jz > nz - 1 ? nz - 1 : jz);
            int64_t j = jx + (int64_t)nx * (jy + (int64_t)ny * jz);
            int event = (j == c) ? face_bc[face] : QSG_ADJ_TRANSIT_ON_PROCESSOR;
            for (int k = 0; k < 4; k++) {
                int f = face * 4 + k;
                hp.facet_event[c * 24 + f] = event;
                hp.facet_adjacent_cell[c * 24 + f] = (int32_t)j;
                bool boundary = (event == QSG_ADJ_BOUNDARY_REFLECTION || event == QSG_ADJ_BOUNDARY_ESCAPE);
                hp.facet_adjacent_facet[c * 24 + f] = boundary ? f : kOpposingFacet[f];
            }
        }
        // cellVolume (MC_Domain.cc:334-355): centre by division
        Vec3 centre{0., 0., 0.};
        for (int p = 0; p < 14; p++) {
            Vec3 v = node(p);
            centre.x += v.x;
            centre.y += v.y;
            centre.z += v.z;
        }
        centre.x /= 14;
        centre.y /= 14;
        centre.z /= 14;
        double volume = 0;
        for (int f = 0; f < 24; f++) {
            Vec3 a = node(kFacetLocalPoints[f][0]), b = node(kFacetLocalPoints[f][1]), cc = node(kFacetLocalPoints[f][2]);
            Vec3 aa{a.x - centre.x, a.y - centre.y, a.z - centre.z};
            Vec3 bb{b.x - centre.x, b.y - centre.y, b.z - centre.z};
            Vec3 ccv{cc.x - centre.x, cc.y - centre.y, cc.z - centre.z};
            Vec3 cr{bb.y * ccv.z - bb.z * ccv.y, bb.z * ccv.x - bb.x * ccv.z, bb.x * ccv.y - bb.y * ccv.x};
            volume += fabs(aa.x * cr.x + aa.y * cr.y + aa.z * cr.z);
        }
        volume /= 6.0;
        hp.cell_volume[c] = volume;
        // cell id: GlobalFccGrid::whichCell of the divided centre (MC_Domain.cc:389-390)
        int wx = (int)(centre.x / dx), wy = (int)(centre.y / dy), wz = (int)(centre.z / dz);
        hp.cell_id[c] = (uint64_t)(wx + (int64_t)nx * (wy + (int64_t)ny * wz)) * UINT64_C(0x0100000000);
        // material: MCT_Cell_Position_3D_G centre (MCT.cc:231-253), last matching geometry wins
        Vec3 pos{0., 0., 0.};
        for (int p = 0; p < 14; p++) {
            Vec3 v = node(p);
            pos.x += v.x;
            pos.y += v.y;
            pos.z += v.z;
        }
        double one_over = 1.0 / ((double)14);
        pos.x *= one_over;
        pos.y *= one_over;
        pos.z *= one_over;
        std::string mat_name;
        for (const GeometrySpec& g : d.geometry)
            if (is_inside(g, pos)) mat_name = g.material;
        if (mat_name.empty()) throw std::runtime_error("deck: a cell centre lies outside every Geometry block");
        int mat = -1;
        for (size_t m = 0; m < hp.material_names.size(); m++)
            if (hp.material_names[m] == mat_name) mat = (int)m;
        if (mat < 0) throw std::runtime_error("deck: Geometry names unknown material '" + mat_name + "'");
        hp.cell_material[c] = mat;
    }
    hp.time_step = s.dt;
}

}  // namespace qsg

extern "C" int qsg_deck_build(const QsgDeck* deck, QsgHostProblem** out)
{
    QSG_API_BEGIN
    if (!deck || !out) return qsg::fail(QSG_ERR_INVALID, "qsg_deck_build: null argument");
    *out = nullptr;
    QsgHostProblem* hp = new QsgHostProblem();
    try {
        qsg::build_problem(deck->deck, *hp);
    } catch (...) {
        delete hp;
        throw;
    }
    *out = hp;
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_host_problem_view(const QsgHostProblem* hp, QsgProblem* v)
{
    if (!hp || !v) return qsg::fail(QSG_ERR_INVALID, "qsg_host_problem_view: null argument");
    memset(v, 0, sizeof(*v));
    v->num_groups = hp->num_groups;
    v->energies = hp->energies.data();
    v->num_isotopes = (int32_t)hp->isotope_reaction_offset.size() - 1;
    v->isotope_reaction_offset = hp->isotope_reaction_offset.data();
    v->reaction_type = hp->reaction_type.data();
    v->reaction_nubar = hp->reaction_nubar.data();
    v->reaction_xs = hp->reaction_xs.data();
    v->num_materials = (int32_t)hp->material_mass.size();
    v->material_isotope_offset = hp->material_isotope_offset.data();
    v->material_isotope_gid = hp->material_isotope_gid.data();
    v->material_atom_fraction = hp->material_atom_fraction.data();
    v->material_mass = hp->material_mass.data();
    v->num_cells = hp->num_cells;
    v->num_nodes = (int32_t)(hp->nodes.size() / 3);
    v->nodes = hp->nodes.data();
    v->cell_points = hp->cell_points.data();
    v->facet_local_points = hp->facet_local_points.data();
    v->facet_planes = hp->facet_planes.data();
    v->facet_event = hp->facet_event.data();
    v->facet_adjacent_cell = hp->facet_adjacent_cell.data();
    v->facet_adjacent_facet = hp->facet_adjacent_facet.data();
    v->cell_material = hp->cell_material.data();
    v->cell_number_density = hp->cell_number_density.data();
    v->cell_volume = hp->cell_volume.data();
    v->cell_id = hp->cell_id.data();
    v->time_step = hp->time_step;
    return QSG_OK;
}

extern "C" int qsg_host_problem_source_rates(const QsgHostProblem* hp, double* rates, int32_t n)
{
    if (!hp || !rates) return qsg::fail(QSG_ERR_INVALID, "qsg_host_problem_source_rates: null argument");
    if (n != (int32_t)hp->material_source_rate.size())
        return qsg::fail(QSG_ERR_INVALID, "qsg_host_problem_source_rates: expected %d materials, got %d",
                         (int)hp->material_source_rate.size(), (int)n);
    for (int32_t i = 0; i < n; i++) rates[i] = hp->material_source_rate[i];
    return QSG_OK;
}

extern "C" int qsg_host_problem_scale_xs(QsgHostProblem* hp, int32_t material, int32_t reaction_type,
                                         int32_t g_lo, int32_t g_hi, double factor)
{
    if (!hp) return qsg::fail(QSG_ERR_INVALID, "qsg_host_problem_scale_xs: null handle");
    if (material < 0 || material >= (int32_t)hp->material_mass.size())
        return qsg::fail(QSG_ERR_INVALID, "qsg_host_problem_scale_xs: material %d out of range", (int)material);
    const int G = hp->num_groups;
    if (g_lo < 0) g_lo = 0;
    if (g_hi > G) g_hi = G;
    for (int k = hp->material_isotope_offset[material]; k < hp->material_isotope_offset[material + 1]; k++) {
        int iso = hp->material_isotope_gid[k];
        for (int r = hp->isotope_reaction_offset[iso]; r < hp->isotope_reaction_offset[iso + 1]; r++) {
            if (hp->reaction_type[r] != reaction_type) continue;
            for (int g = g_lo; g < g_hi; g++) hp->reaction_xs[(int64_t)r * G + g] *= factor;
        }
    }
    return QSG_OK;
}

extern "C" int qsg_host_problem_free(QsgHostProblem* hp)
{
    delete hp;
    return QSG_OK;
}
