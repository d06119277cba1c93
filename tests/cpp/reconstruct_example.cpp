// The reconstruction flow of the reference's main (mainReconstruct.cpp) on
// the drop-in headers, with no VTK: geometry file -> DICOM series ->
// log(1 + x) -> first backprojection -> ART (or MLEM) with the per-iteration
// dumps -> float and 16-bit TIFFs.
//
// usage: reconstruct_example <geometry.xml> <dicom dir> <result dir/> [art|mlem] [iterations]
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "kevernals_dicom.hpp"
#include "kevernals_output.hpp"
#include "kevernals_tomo.hpp"

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s <geometry.xml> <dicom dir> <result dir/> [art|mlem] [iterations]\n", argv[0]);
        return 2;
    }
    const std::string resultDir = argv[3];
    const bool mlem = argc > 4 && std::string(argv[4]) == "mlem";
    const int iterations = argc > 5 ? std::atoi(argv[5]) : 5;

    auto geometry = std::make_unique<TomoGeometry>(std::string(argv[1]));
    if (!geometry->IsValid()) {
        std::cout << "invalid geometry: " << geometry->ErrorMessage() << std::endl;
        return 1;
    }
    std::cout << *geometry << std::endl;

    DICOMReader reader(geometry.get());
    auto data = reader.ReadDirectory(argv[2], {});
    if (data.has_error()) {
        std::cout << PrintErrorCode(data.error(), reader.LastError()) << std::endl;
        return 1;
    }
    auto projections = LogarithmicScale(data.value());
    WriteTIFF(resultDir + "projectionImages.tiff", projections);

    auto first = recons::BackProjection(geometry.get(), projections);
    if (first.has_error()) {
        std::cout << PrintErrorCode(first.error()) << std::endl;
        return 1;
    }
    auto result = mlem ? recons::MLEM(geometry.get(), projections, iterations, 0.5F, first.value(), resultDir)
                       : recons::ART(geometry.get(), projections, iterations, 0.5F, first.value(), resultDir);
    if (result.has_error()) {
        std::cout << PrintErrorCode(result.error()) << std::endl;
        return 1;
    }
    const std::string name = mlem ? "MLEMReconstructedImage" : "ARTReconstructedImage";
    if (!WriteTIFF(resultDir + name + ".tiff", result.value())) return 1;
    auto u16 = RescaleToUInt16(result.value());
    HistUniformization16Bit(u16);
    if (!WriteTIFF(resultDir + name + "_u16.tiff", u16)) return 1;
    std::cout << "done" << std::endl;
    return 0;
}
