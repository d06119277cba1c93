// Minimal stand-in for VTK's vtkImageData (TEST INFRASTRUCTURE, used only by
// oracle/build_ref.sh to compile parts of the reference that take images:
// commons/HistogramMatchingTools.h, modules/dataHandling/PhantomMaker.cpp and
// the ART / MLEM drivers of modules/reconstruction/Reconstructors.h).  One
// scalar component of VTK_FLOAT or VTK_UNSIGNED_SHORT, x fastest, the whole
// extent starting at 0.
#pragma once

#include <cstddef>
#include <vector>

#define VTK_UNSIGNED_SHORT 5
#define VTK_FLOAT 10

class vtkImageData {
public:
    static vtkImageData *New() { return new vtkImageData; }
    void SetDimensions(int x, int y, int z) {
        m_dims[0] = x;
        m_dims[1] = y;
        m_dims[2] = z;
    }
    int *GetDimensions() { return m_dims; }
    void SetSpacing(double x, double y, double z) {
        m_spacing[0] = x;
        m_spacing[1] = y;
        m_spacing[2] = z;
    }
    double *GetSpacing() { return m_spacing; }
    int *GetExtent() {
        for (int i = 0; i < 3; ++i) {
            m_extent[2 * i] = 0;
            m_extent[2 * i + 1] = m_dims[i] - 1;
        }
        return m_extent;
    }
    void AllocateScalars(int type, int /*components*/) {
        m_type = type;
        m_bytes.assign(count() * element(), 0);
    }
    int GetScalarType() const { return m_type; }
    void *GetScalarPointer() { return m_bytes.data(); }
    void *GetScalarPointer(int x, int y, int z) {
        return m_bytes.data() + ((static_cast<size_t>(z) * m_dims[1] + y) * m_dims[0] + x) * element();
    }
    void Modified() {}

private:
    size_t count() const { return static_cast<size_t>(m_dims[0]) * m_dims[1] * m_dims[2]; }
    size_t element() const { return m_type == VTK_FLOAT ? 4 : 2; }
    int m_dims[3] = {0, 0, 0};
    int m_extent[6] = {0, -1, 0, -1, 0, -1};
    double m_spacing[3] = {1, 1, 1};
    int m_type = VTK_UNSIGNED_SHORT;
    std::vector<unsigned char> m_bytes;
};
