// Runs the reference's own histogram tools (source/commons/
// HistogramMatchingTools.h, compiled from the reference tree by
// oracle/build_ref.sh against the VTK stand-ins in ref_vtk_stub/) on a raw
// unsigned-short volume and writes their results as raw files:
//   ref_histogram <u16.raw> nx ny nz <out_dir/>
//   -> hist.raw (GetHist16Bit, 65536 int32), uniform.raw
//      (HistUniformization16Bit), halftop.raw (HistHalfTop16Bit)
// TEST INFRASTRUCTURE: the checker for include/kevernals_output.hpp.
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "commons/HistogramMatchingTools.h"

static vtkSmartPointer<vtkImageData> load(const std::vector<unsigned short> &v, int nx, int ny, int nz) {
    auto im = vtkSmartPointer<vtkImageData>::New();
    im->SetDimensions(nx, ny, nz);
    im->AllocateScalars(VTK_UNSIGNED_SHORT, 1);
    std::memcpy(im->GetScalarPointer(), v.data(), v.size() * sizeof(unsigned short));
    return im;
}

static void save(const std::string &path, const void *p, size_t bytes) {
    std::ofstream(path, std::ios::binary).write(static_cast<const char *>(p), static_cast<std::streamsize>(bytes));
}

int main(int argc, char **argv) {
    if (argc != 6) return 2;
    const int nx = std::atoi(argv[2]), ny = std::atoi(argv[3]), nz = std::atoi(argv[4]);
    const std::string out = argv[5];
    std::vector<unsigned short> v(static_cast<size_t>(nx) * ny * nz);
    std::ifstream(argv[1], std::ios::binary).read(reinterpret_cast<char *>(v.data()),
                                                  static_cast<std::streamsize>(v.size() * 2));
    const auto hist = GetHist16Bit(load(v, nx, ny, nz));
    save(out + "hist.raw", hist.data(), hist.size() * sizeof(int));
    auto uni = load(v, nx, ny, nz);
    HistUniformization16Bit(uni);
    save(out + "uniform.raw", uni->GetScalarPointer(), v.size() * 2);
    auto half = load(v, nx, ny, nz);
    HistHalfTop16Bit(half);
    save(out + "halftop.raw", half->GetScalarPointer(), v.size() * 2);
    return 0;
}
