// Compile-only stand-in for VTK's vtkImageAppend (TEST INFRASTRUCTURE), see
// vtk_unused_filter.h.
#pragma once

#include "vtk_unused_filter.h"

class vtkImageAppend : public vtkUnusedFilter {
public:
    static vtkImageAppend *New() { return new vtkImageAppend; }
};
