// Drives the C++ drop-in API (include/kevernals_tomo.hpp) the way the
// reference's callers do (mainReconstruct.cpp: Projector, recons::MLEM / ART /
// BackProjection / ShiftAndAdd) and writes every result as raw float32 for
// tests/test_gpu_dropin.py to compare with the oracle.
//
// usage: test_dropin <case.bin> <out_dir/>
// case.bin: int32 nx ny nz nu nv P; float32 dx dy dz du dv fulcrum_z det_z;
//           float32 src[P][3]; float32 roi_bl[P][2]; float32 vol[nz][ny][nx];
//           float32 proj[P][nv][nu]
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "kevernals_tomo.hpp"

static void dump(const std::string &path, const ImageDataPtr &img) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char *>(img->data()), (std::streamsize)(img->size() * 4));
}

static ImageDataPtr image(int x, int y, int z, const float *src) {
    auto im = ImageData::New();
    im->SetDimensions(x, y, z);
    im->AllocateScalars();
    std::copy(src, src + im->size(), im->data());
    return im;
}

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    int32_t hdr[6];
    float fl[7];
    in.read(reinterpret_cast<char *>(hdr), sizeof hdr);
    in.read(reinterpret_cast<char *>(fl), sizeof fl);
    const int nx = hdr[0], ny = hdr[1], nz = hdr[2], nu = hdr[3], nv = hdr[4], P = hdr[5];
    std::vector<float> src(3 * P), bl(2 * P), vol((size_t)nx * ny * nz), proj((size_t)P * nu * nv);
    in.read(reinterpret_cast<char *>(src.data()), src.size() * 4);
    in.read(reinterpret_cast<char *>(bl.data()), bl.size() * 4);
    in.read(reinterpret_cast<char *>(vol.data()), vol.size() * 4);
    in.read(reinterpret_cast<char *>(proj.data()), proj.size() * 4);
    if (!in) return 3;
    std::vector<Position3D> sources;
    std::vector<Position2D> origins;
    for (int i = 0; i < P; ++i) {
        sources.push_back({src[3 * i], src[3 * i + 1], src[3 * i + 2]});
        origins.push_back({bl[2 * i], bl[2 * i + 1]});
    }
    TomoGeometry geom({nx, ny, nz}, {fl[0], fl[1], fl[2]}, sources, origins, fl[6], {nu, nv}, {fl[3], fl[4]},
                      {0.f, 0.f, fl[5]});
    const std::string out = argv[2];

    auto volume = image(nx, ny, nz, vol.data());
    auto projections = image(nu, nv, P, proj.data());

    Projector projector{&geom};
    auto fwd = projector.PerformProjection(volume);
    if (!fwd) return 4;
    dump(out + "rc_fwd.raw", fwd);
    auto back = recons::BackProjection(&geom, fwd);
    if (!back) return 5;
    dump(out + "rc_back.raw", back.value());

    auto x = image(nx, ny, nz, std::vector<float>(vol.size(), 1.f).data());
    auto mlem = recons::MLEM(&geom, projections, 3, 0.5f, x, std::nullopt);
    if (!mlem || mlem.value() != x) return 6;   // the initial volume is updated in place
    dump(out + "rc_mlem.raw", mlem.value());
    auto art = recons::ART(&geom, projections, 3, 0.5f, std::nullopt, std::nullopt);
    if (!art) return 7;
    dump(out + "rc_art.raw", art.value());
    auto saa = recons::ShiftAndAdd(&geom, projections, std::nullopt);
    if (!saa) return 8;
    dump(out + "rc_saa.raw", saa.value());

    Projector exact{&geom, KV_FAMILY_EXACT};
    auto efwd = exact.PerformProjection(volume);
    if (!efwd) return 9;
    dump(out + "exact_fwd.raw", efwd);

    auto single = ImageData::New();
    projector.PerformProjection(volume, sources[0], single);
    dump(out + "rc_single.raw", single);

    auto fbp = recons::FilteredBackProjection(&geom, efwd, 16);
    if (!fbp) return 12;
    dump(out + "exact_fbp.raw", fbp.value());
    // verbose mode: TIFF dumps of the initial volume and every iterate
    auto xv = image(nx, ny, nz, std::vector<float>(vol.size(), 1.f).data());
    auto verbose = recons::MLEM(&geom, projections, 2, 0.5f, xv, out + "verbose_");
    if (!verbose) return 13;

    // error convention: a null initial volume is reported, not fatal
    auto bad = recons::MLEM(&geom, projections, 1, 1.f, ImageDataPtr{}, std::nullopt);
    if (bad || bad.error() != ReconstructorsErrorCode::ART) return 10;
    auto bad2 = recons::ShiftAndAdd(&geom, ImageDataPtr{}, std::nullopt);
    if (bad2.error() != ReconstructorsErrorCode::ShiftAndAdd) return 11;
    std::printf("dropin ok\n");
    return 0;
}
