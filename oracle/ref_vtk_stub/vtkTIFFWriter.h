// Compile-only stand-in for VTK's vtkTIFFWriter (TEST INFRASTRUCTURE), see
// vtk_unused_filter.h.
#pragma once

#include "vtk_unused_filter.h"

class vtkTIFFWriter : public vtkUnusedFilter {
public:
    static vtkTIFFWriter *New() { return new vtkTIFFWriter; }
};
