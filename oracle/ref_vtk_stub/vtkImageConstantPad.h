// Compile-only stand-in for VTK's vtkImageConstantPad (TEST INFRASTRUCTURE), see
// vtk_unused_filter.h.
#pragma once

#include "vtk_unused_filter.h"

class vtkImageConstantPad : public vtkUnusedFilter {
public:
    static vtkImageConstantPad *New() { return new vtkImageConstantPad; }
};
