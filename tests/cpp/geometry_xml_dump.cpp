// Reads a geometry file with the drop-in header's TomoGeometry(path) and
// prints the flattened description the kernels receive, as JSON.  With
// "adapt i j ..." after the path it first applies
// PerformCheatingAdaptationsForDemonstration({i, j, ...}); with "accessors"
// as the last argument it prints the geometry accessors instead, with
// "views" whether the part views (GetVolume, ...) agree with them.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "kevernals_tomo.hpp"

// a string as the body of a JSON string literal
static std::string json_escape(const std::string &v) {
    std::string out;
    for (char c : v) {
        if (c == '"' || c == '\\') out += '\\';
        out += c;
    }
    return out;
}

static void floats(const char *key, const std::vector<float> &v, bool last = false) {
    std::printf("\"%s\": [", key);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.9g", i ? ", " : "", v[i]);
    std::printf("]%s", last ? "" : ", ");
}

static int accessors(const TomoGeometry &g) {
    // the position lists only when small (an adapted detector has 3048^2 pixels per view)
    std::vector<float> grid, pos, rpos;
    const auto det_n = g.projectionsPositionsIndices().size();
    const auto roi_n = g.projectionsRoisPositionsIndices().size();
    for (const auto &p : g.volumeGridPositions()) grid.insert(grid.end(), {p.x, p.y, p.z});
    if (det_n <= 100000)
        for (const auto &p : g.projectionsPositions()) pos.insert(pos.end(), {p.x, p.y});
    if (roi_n <= 100000)
        for (const auto &p : g.projectionsRoisPositions()) rpos.insert(rpos.end(), {p.x, p.y});
    const auto w = g.volumeWSize3D(), b = g.volumeBLF(), t = g.volumeTRB();
    const auto dw = g.projectionsWSize(), rw = g.projectionsRoisWSize();
    const auto ds = g.projectionsSize(), rs = g.projectionsRoisSize();
    const auto dp = g.projectionsPixelSpacing(), rp = g.projectionsRoisPixelSpacing();
    std::printf("{");
    floats("wsize", {w.x, w.y, w.z});
    floats("blf", {b.x, b.y, b.z});
    floats("trb", {t.x, t.y, t.z});
    floats("volume_size", {g.volumeSize()});
    floats("xs", g.volumeXs());
    floats("ys", g.volumeYs());
    floats("zs", g.volumeZs());
    floats("grid", grid);
    floats("det_wsize", {dw.x, dw.y});
    floats("det_pitch", {dp.x, dp.y});
    floats("roi_wsize", {rw.x, rw.y});
    floats("roi_pitch", {rp.x, rp.y});
    std::vector<float> dbl;
    for (const auto &p : g.projectionsBottomLeftPositions()) dbl.insert(dbl.end(), {p.x, p.y});
    floats("det_bl", dbl);
    floats("det_x1", g.projectionsXPositions().at(1));
    floats("det_y1", g.projectionsYPositions().at(1));
    floats("roi_x1", g.projectionsRoisXPositions().at(1));
    floats("roi_y1", g.projectionsRoisYPositions().at(1));
    floats("det_positions", pos);
    floats("roi_positions", rpos);
    std::printf("\"det_size\": [%d, %d], \"roi_size\": [%d, %d], \"n_voxel_indices\": %zu, "
                "\"n_det_indices\": %zu, \"n_roi_indices\": %zu, \"last_voxel_index\": %d}\n",
                ds.x, ds.y, rs.x, rs.y, g.volumeVoxelsIndices().size(), det_n, roi_n,
                g.volumeVoxelsIndices().back());
    return 0;
}

template <typename A, typename B> static bool same(const A &a, const B &b) { return a == b; }
static bool same(const Position2D &a, const Position2D &b) { return a.x == b.x && a.y == b.y; }
static bool same(const Position3D &a, const Position3D &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
static bool same(const Size2D &a, const Size2D &b) { return a.x == b.x && a.y == b.y; }
static bool same(const Size3D &a, const Size3D &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
static bool same(const PixelSpacing &a, const PixelSpacing &b) { return a.x == b.x && a.y == b.y; }
static bool same(const VoxelSpacing &a, const VoxelSpacing &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <typename T> static bool same(const std::vector<T> &a, const std::vector<T> &b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (!same(a[i], b[i])) return false;
    return true;
}

// The part views (GetVolume / GetProjections / GetProjectionsRois /
// GetTable) against the geometry's own accessors, printed as JSON booleans.
static int views(const TomoGeometry &g) {
    const TomoVolume *v = g.GetVolume();
    const TomoProjectionsSet *d = g.GetProjections(), *r = g.GetProjectionsRois();
    const TomoTable *t = g.GetTable();
    const Size3D n = g.volumeSize3D();
    const bool vol = v->GetVoxelsNumber() == n.x * n.y * n.z && v->GetSize() == g.volumeSize() &&
                     same(v->GetSize3D(), n) && same(v->GetWSize3D(), g.volumeWSize3D()) &&
                     same(v->GetBottomLeftFront(), g.volumeBLF()) && same(v->GetTopRightBack(), g.volumeTRB()) &&
                     same(v->GetVoxelSpacing(), g.volumeVoxelSpacing()) && same(v->GetXPositions(), g.volumeXs()) &&
                     same(v->GetYPositions(), g.volumeYs()) && same(v->GetZPositions(), g.volumeZs()) &&
                     same(v->GetGridPositions(), g.volumeGridPositions()) &&
                     same(v->GetVoxelsIndices(), g.volumeVoxelsIndices());
    const bool det = same(d->GetBottomLeftPositions(), g.projectionsBottomLeftPositions()) &&
                     same(d->GetSize(), g.projectionsSize()) && same(d->GetWSize(), g.projectionsWSize()) &&
                     same(d->GetPixelSpacing(), g.projectionsPixelSpacing()) &&
                     same(d->GetXPositions(), g.projectionsXPositions()) &&
                     same(d->GetYPositions(), g.projectionsYPositions()) &&
                     d->GetNProjections() == g.nbProjections();
    const bool roi = same(r->GetBottomLeftPositions(), g.projectionsRoisBottomLeftPositions()) &&
                     same(r->GetSize(), g.projectionsRoisSize()) && same(r->GetWSize(), g.projectionsRoisWSize()) &&
                     same(r->GetPixelSpacing(), g.projectionsRoisPixelSpacing()) &&
                     same(r->GetXPositions(), g.projectionsRoisXPositions()) &&
                     same(r->GetYPositions(), g.projectionsRoisYPositions()) &&
                     same(r->GetProjectionPositions(), g.projectionsRoisPositions()) &&
                     same(r->GetProjectionPixelsIndices(), g.projectionsRoisPositionsIndices()) &&
                     r->GetNProjections() == g.nbProjectionsRois();
    const bool tab = t->GetSourcesNumber() == g.nbProjections() &&
                     same(t->GetSourcesYPositions(), g.sourcesYPositions()) &&
                     t->GetSourcesXCommonPosition() == g.sourcesXCommonPosition() &&
                     t->GetSourcesZCommonPosition() == g.sourcesZCommonPosition() &&
                     t->GetDetectorsZCommonPosition() == g.detectorsZCommonPosition();
    std::printf("{\"volume\": %s, \"projections\": %s, \"rois\": %s, \"table\": %s, \"voxels\": %d, "
                "\"views\": %d}\n",
                vol ? "true" : "false", det ? "true" : "false", roi ? "true" : "false", tab ? "true" : "false",
                v->GetVoxelsNumber(), d->GetNProjections());
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    TomoGeometry geo{std::string(argv[1])};
    if (!geo.IsValid()) {
        std::printf("{\"valid\": false, \"error\": \"%s\"}\n", json_escape(geo.ErrorMessage()).c_str());
        return 0;
    }
    const bool show_accessors = std::string(argv[argc - 1]) == "accessors";
    const bool show_views = std::string(argv[argc - 1]) == "views";
    if (argc > 2 && std::string(argv[2]) == "adapt") {
        std::vector<int> remove;
        for (int i = 3; i < argc - (show_accessors || show_views ? 1 : 0); ++i) remove.push_back(std::atoi(argv[i]));
        geo.PerformCheatingAdaptationsForDemonstration(remove);
    }
    if (show_accessors) return accessors(geo);
    if (show_views) return views(geo);
    const auto f = geo.flatten();
    const kv_geometry &g = f->g;
    std::printf("{\"valid\": true, \"n\": [%d, %d, %d], \"d\": [%.9g, %.9g, %.9g], \"views\": %d, "
                "\"det\": [%d, %d], \"pitch\": [%.9g, %.9g], \"fulcrum_z\": %.9g, \"src\": [",
                g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.n_views, g.nu, g.nv, g.du, g.dv, g.fulcrum_z);
    for (int i = 0; i < 3 * g.n_views; ++i) std::printf("%s%.9g", i ? ", " : "", g.src[i]);
    std::printf("], \"det_origin\": [");
    for (int i = 0; i < 3 * g.n_views; ++i) std::printf("%s%.9g", i ? ", " : "", g.det_origin[i]);
    std::printf("]}\n");
    return 0;
}
