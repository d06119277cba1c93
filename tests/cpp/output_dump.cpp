// Output tools of the drop-in on a float32 volume read from a raw file:
// writes vol.tif, u16.tif and uniform.tif, and the 16-bit images as raw
// files (u16.raw, uniform.raw, halftop.raw) for comparison.
#include <cstdio>
#include <cstdlib>
#include <fstream>

#include "kevernals_output.hpp"

static void dump(const std::string &p, const ImageU16Ptr &im) {
    std::ofstream f(p, std::ios::binary);
    f.write(reinterpret_cast<const char *>(im->data.data()), (std::streamsize)(im->size() * 2));
}

int main(int argc, char **argv) {
    if (argc < 6) return 2;
    const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]);
    const std::string out = argv[5];
    auto vol = ImageData::New();
    vol->SetDimensions(nx, ny, nz);
    vol->AllocateScalars();
    std::ifstream f(argv[1], std::ios::binary);
    f.read(reinterpret_cast<char *>(vol->data()), (std::streamsize)(vol->size() * 4));
    if (!WriteTIFF(out + "/vol.tif", vol)) return 3;
    auto u = RescaleToUInt16(vol);
    dump(out + "/u16.raw", u);
    if (!WriteTIFF(out + "/u16.tif", u)) return 3;
    auto uni = std::make_shared<ImageU16>(*u);
    HistUniformization16Bit(uni);
    dump(out + "/uniform.raw", uni);
    if (!WriteTIFF(out + "/uniform.tif", uni)) return 3;
    auto half = std::make_shared<ImageU16>(*u);
    HistHalfTop16Bit(half);
    dump(out + "/halftop.raw", half);
    std::printf("ok\n");
    return 0;
}
