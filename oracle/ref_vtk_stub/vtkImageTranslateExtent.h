// Compile-only stand-in for VTK's vtkImageTranslateExtent (TEST INFRASTRUCTURE), see
// vtk_unused_filter.h.
#pragma once

#include "vtk_unused_filter.h"

class vtkImageTranslateExtent : public vtkUnusedFilter {
public:
    static vtkImageTranslateExtent *New() { return new vtkImageTranslateExtent; }
};
