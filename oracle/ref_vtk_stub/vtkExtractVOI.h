// Compile-only stand-in for VTK's vtkExtractVOI (TEST INFRASTRUCTURE), see
// vtk_unused_filter.h.
#pragma once

#include "vtk_unused_filter.h"

class vtkExtractVOI : public vtkUnusedFilter {
public:
    static vtkExtractVOI *New() { return new vtkExtractVOI; }
};
