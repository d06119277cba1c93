// Minimal stand-in for VTK's vtkImageData (TEST INFRASTRUCTURE, used only by
// oracle/build_ref.sh to compile the reference's
// commons/HistogramMatchingTools.h, which needs nothing else from VTK):
// an image of unsigned shorts with its dimensions, its scalar type and
// voxel addressing, x fastest.
#pragma once

#include <cstddef>
#include <vector>

#define VTK_UNSIGNED_SHORT 5

class vtkImageData {
public:
    static vtkImageData *New() { return new vtkImageData; }
    void SetDimensions(int x, int y, int z) {
        m_dims[0] = x;
        m_dims[1] = y;
        m_dims[2] = z;
        m_data.assign(static_cast<size_t>(x) * y * z, 0);
    }
    int *GetDimensions() { return m_dims; }
    int GetScalarType() const { return VTK_UNSIGNED_SHORT; }
    void *GetScalarPointer() { return m_data.data(); }
    void *GetScalarPointer(int x, int y, int z) {
        return m_data.data() + (static_cast<size_t>(z) * m_dims[1] + y) * m_dims[0] + x;
    }

private:
    int m_dims[3] = {0, 0, 0};
    std::vector<unsigned short> m_data;
};
