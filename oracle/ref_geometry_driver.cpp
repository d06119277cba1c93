// Reads a geometry file with the reference's own reader
// (source/modules/geometry/TomoGeometry.cpp with the vendored tinyxml2),
// compiled from the reference tree by oracle/build_ref.sh, and prints, as the
// last line of its output, one JSON object with the fields that
// tests/cpp/geometry_xml_dump.cpp prints for the drop-in's reader:
//   default      what Projector::PerformProjection hands its kernels
//                (Projector.cu:877-940): volume size and spacing, views,
//                ROI size, detector pitch, the fulcrum height, per-view
//                sources (common x, y_i, common z) and ROI corners on the
//                common detector plane;
//   accessors    the value accessors of TomoGeometry.h:34-89.
// "adapt i j ..." after the path first applies
// PerformCheatingAdaptationsForDemonstration({i, j, ...}).  The reference
// prints its own messages on stdout too, hence "last line".
// TEST INFRASTRUCTURE: the checker for the drop-in's XML reader.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "modules/geometry/TomoGeometry.h"

static void floats(const char *key, const std::vector<float> &v, bool last = false) {
    std::printf("\"%s\": [", key);
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.9g", i ? ", " : "", v[i]);
    std::printf("]%s", last ? "" : ", ");
}

static void flat(const TomoGeometry &g) {
    const auto n = g.volumeSize3D();
    const auto d = g.volumeVoxelSpacing();
    const auto roi = g.projectionsRoisSize();
    const auto px = g.projectionsPixelSpacing();
    const int views = g.nbProjectionsRois();
    std::vector<float> src, det;
    for (int i = 0; i < views; ++i) {
        src.insert(src.end(), {g.sourcesXCommonPosition(), g.sourcesYPositions().at(i), g.sourcesZCommonPosition()});
        const auto b = g.projectionsRoisBottomLeftPositions().at(i);
        det.insert(det.end(), {b.x, b.y, g.detectorsZCommonPosition()});
    }
    std::printf("\n{\"valid\": true, \"n\": [%d, %d, %d], \"d\": [%.9g, %.9g, %.9g], \"views\": %d, "
                "\"det\": [%d, %d], \"pitch\": [%.9g, %.9g], \"fulcrum_z\": %.9g, ",
                n.x, n.y, n.z, d.x, d.y, d.z, views, roi.x, roi.y, px.x, px.y, g.fulcrum().z);
    floats("src", src);
    floats("det_origin", det, true);
    std::printf("}\n");
}

static void accessors(const TomoGeometry &g) {
    std::vector<float> grid, pos, rpos, dbl;
    const auto det_n = g.projectionsPositionsIndices().size();
    const auto roi_n = g.projectionsRoisPositionsIndices().size();
    for (const auto &p : g.volumeGridPositions()) grid.insert(grid.end(), {p.x, p.y, p.z});
    if (det_n <= 100000)
        for (const auto &p : g.projectionsPositions()) pos.insert(pos.end(), {p.x, p.y});
    if (roi_n <= 100000)
        for (const auto &p : g.projectionsRoisPositions()) rpos.insert(rpos.end(), {p.x, p.y});
    for (const auto &p : g.projectionsBottomLeftPositions()) dbl.insert(dbl.end(), {p.x, p.y});
    const auto w = g.volumeWSize3D();
    const auto b = g.volumeBLF();
    const auto t = g.volumeTRB();
    const auto dw = g.projectionsWSize();
    const auto rw = g.projectionsRoisWSize();
    const auto ds = g.projectionsSize();
    const auto rs = g.projectionsRoisSize();
    const auto dp = g.projectionsPixelSpacing();
    const auto rp = g.projectionsRoisPixelSpacing();
    std::printf("\n{");
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
    floats("det_bl", dbl);
    floats("det_x1", g.projectionsXPositions().at(1));
    floats("det_y1", g.projectionsYPositions().at(1));
    floats("roi_x1", g.projectionsRoisXPositions().at(1));
    floats("roi_y1", g.projectionsRoisYPositions().at(1));
    floats("det_positions", pos);
    floats("roi_positions", rpos);
    const auto vox = g.volumeVoxelsIndices();
    std::printf("\"det_size\": [%d, %d], \"roi_size\": [%d, %d], \"n_voxel_indices\": %zu, "
                "\"n_det_indices\": %zu, \"n_roi_indices\": %zu, \"last_voxel_index\": %d}\n",
                ds.x, ds.y, rs.x, rs.y, vox.size(), det_n, roi_n, vox.back());
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    TomoGeometry geo{std::string(argv[1])};
    if (!geo.IsValid()) {
        std::printf("\n{\"valid\": false}\n");
        return 0;
    }
    const bool show_accessors = std::string(argv[argc - 1]) == "accessors";
    if (argc > 2 && std::string(argv[2]) == "adapt") {
        std::vector<int> remove;
        for (int i = 3; i < argc - (show_accessors ? 1 : 0); ++i) remove.push_back(std::atoi(argv[i]));
        geo.PerformCheatingAdaptationsForDemonstration(remove);
    }
    if (show_accessors) accessors(geo);
    else flat(geo);
    return 0;
}
