// Stand-in for the reference's modules/reconstruction/Projector.h (TEST
// INFRASTRUCTURE, used only by oracle/build_ref.sh for the driver checker):
// the reference's public Projector interface, backed by the reference's own
// projector kernels compiled for the host (oracle/_ref/libkvref.so:
// kvref_forward / kvref_back run CudaPerformProjection and
// CudaPerformBackProjection, Projector.cu:227-785, per ray and per voxel).
// The geometry is flattened as Projector::PerformProjection does
// (Projector.cu:877-940: common source x and z, per-view source y, ROI
// corners on the common detector plane, detector pitch) and the outputs are
// shaped as there (:965-969 and :1136-1140).  The device allocations and
// copies of the reference's wrappers have no counterpart on the host.
#pragma once

#include <cstdint>
#include <vector>

#include "commons/ImageDataPtr.h"
#include "modules/geometry/TomoGeometry.h"

extern "C" {
struct kvref_geom {
    int32_t nx, ny, nz;
    float dx, dy, dz;
    int32_t n_views;
    int32_t nu, nv;
    float du, dv;
    const float *src;
    const float *det_origin;
    float fulcrum_z;
};
void kvref_forward(const kvref_geom *g, const float *vol, float *proj);
void kvref_back(const kvref_geom *g, const float *proj, float *vol);
}

class Projector {
public:
    Projector(TomoGeometry *p_tomoGeometry) : m_tomoGeometry{p_tomoGeometry} {}

    vtkSmartPointer<vtkImageData> PerformProjection(vtkSmartPointer<vtkImageData> p_volume) const {
        Flat f = flatten();
        auto out = vtkSmartPointer<vtkImageData>::New();
        out->SetDimensions(f.g.nu, f.g.nv, f.g.n_views);
        out->SetSpacing(f.g.du, f.g.dv, 1.);
        out->AllocateScalars(VTK_FLOAT, 1);
        kvref_forward(&f.g, static_cast<const float *>(p_volume->GetScalarPointer()),
                      static_cast<float *>(out->GetScalarPointer()));
        return out;
    }

    // unfinished in the reference (Projector.cu:823-870): no effect
    void PerformProjection(const vtkSmartPointer<vtkImageData>, const Position3D &,
                           vtkSmartPointer<vtkImageData>) const {}

    vtkSmartPointer<vtkImageData> PerformBackProjection(vtkSmartPointer<vtkImageData> p_projections) const {
        Flat f = flatten();
        auto out = vtkSmartPointer<vtkImageData>::New();
        out->SetDimensions(f.g.nx, f.g.ny, f.g.nz);
        out->SetSpacing(f.g.dx, f.g.dy, f.g.dz);
        out->AllocateScalars(VTK_FLOAT, 1);
        kvref_back(&f.g, static_cast<const float *>(p_projections->GetScalarPointer()),
                   static_cast<float *>(out->GetScalarPointer()));
        return out;
    }

private:
    struct Flat {
        kvref_geom g;
        std::vector<float> src, det;
    };
    Flat flatten() const {
        const TomoGeometry &t = *m_tomoGeometry;
        Flat f;
        const auto n = t.GetVolume()->GetSize3D();
        const auto d = t.GetVolume()->GetVoxelSpacing();
        const auto roi = t.projectionsRoisSize();
        const auto px = t.projectionsPixelSpacing();
        const int views = t.nbProjectionsRois();
        const auto ys = t.sourcesYPositions();
        const auto bl = t.projectionsRoisBottomLeftPositions();
        for (int i = 0; i < views; ++i) {
            f.src.insert(f.src.end(), {t.sourcesXCommonPosition(), ys.at(i), t.sourcesZCommonPosition()});
            f.det.insert(f.det.end(), {bl.at(i).x, bl.at(i).y, t.detectorsZCommonPosition()});
        }
        f.g = kvref_geom{n.x, n.y, n.z, d.x, d.y, d.z, views, roi.x, roi.y, px.x, px.y,
                         f.src.data(), f.det.data(), t.fulcrum().z};
        return f;
    }
    TomoGeometry *m_tomoGeometry;
};
