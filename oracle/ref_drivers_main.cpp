// Runs the reference's own ART and MLEM drivers (recons::ART / recons::MLEM,
// source/modules/reconstruction/Reconstructors.h:19-253, compiled from the
// reference tree by oracle/build_ref.sh) on a geometry file read by the
// reference's reader and a raw float32 projection stack [P][nv][nu], from the
// reference's uniform start (PhantomMaker, background 1), on the reference's
// kernels compiled for the host (the Projector stand-in in ref_driver_shim/):
//   ref_drivers <geometry.xml> <proj.raw> <mlem|art> <iterations> <relax> <out.raw>
// writes the reconstructed volume [nz][ny][nx] as raw float32;
//   ref_drivers <geometry.xml> saa-shifts
// runs recons::ShiftAndAdd (Reconstructors.h:263-379) over VTK filter
// stand-ins that record the integer row shift the reference computes for
// every slice and view and prints them, slice-major, as the last line of
// output ({"status": "error"} when the reference refuses the geometry).
// TEST INFRASTRUCTURE: the checker for the restated drivers of the oracle.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>

#include "modules/reconstruction/Reconstructors.h"

int main(int argc, char **argv) {
    if (argc != 7 && !(argc == 3 && std::string(argv[2]) == "saa-shifts")) return 2;
    TomoGeometry geometry{std::string(argv[1])};
    if (!geometry.IsValid()) return 3;
    const auto roi = geometry.projectionsRoisSize();
    auto projections = vtkSmartPointer<vtkImageData>::New();
    projections->SetDimensions(roi.x, roi.y, geometry.nbProjectionsRois());
    projections->AllocateScalars(VTK_FLOAT, 1);
    if (argc == 3) {
        auto r = recons::ShiftAndAdd(&geometry, projections, std::nullopt);
        if (r.has_error()) {
            std::printf("\n{\"status\": \"error\"}\n");
            return 0;
        }
        std::printf("\n{\"status\": \"ok\", \"shifts\": [");
        for (size_t i = 0; i < vtk_recorded_shifts.size(); ++i) std::printf("%s%d", i ? ", " : "", vtk_recorded_shifts[i]);
        std::printf("]}\n");
        return 0;
    }
    const size_t n = static_cast<size_t>(roi.x) * roi.y * geometry.nbProjectionsRois();
    std::ifstream(argv[2], std::ios::binary)
        .read(static_cast<char *>(projections->GetScalarPointer()), static_cast<std::streamsize>(n * 4));
    const bool mlem = std::string(argv[3]) == "mlem";
    const int iterations = std::atoi(argv[4]);
    const float relax = static_cast<float>(std::atof(argv[5]));
    auto result = mlem ? recons::MLEM(&geometry, projections, iterations, relax, std::nullopt, std::nullopt)
                       : recons::ART(&geometry, projections, iterations, relax, std::nullopt, std::nullopt);
    if (result.has_error()) return 4;
    auto volume = result.value();
    const int *d = volume->GetDimensions();
    std::ofstream(argv[6], std::ios::binary)
        .write(static_cast<const char *>(volume->GetScalarPointer()),
               static_cast<std::streamsize>(static_cast<size_t>(d[0]) * d[1] * d[2] * 4));
    return 0;
}
