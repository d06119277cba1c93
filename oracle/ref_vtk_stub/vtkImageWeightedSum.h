// Compile-only stand-in for VTK's vtkImageWeightedSum (TEST INFRASTRUCTURE), see
// vtk_unused_filter.h.
#pragma once

#include "vtk_unused_filter.h"

class vtkImageWeightedSum : public vtkUnusedFilter {
public:
    static vtkImageWeightedSum *New() { return new vtkImageWeightedSum; }
};
