// Stand-in for VTK's vtkImageConstantPad (TEST INFRASTRUCTURE), see vtk_recording_filter.h.
#pragma once

#include "vtk_recording_filter.h"

class vtkImageConstantPad : public vtkRecordingFilter {
public:
    static vtkImageConstantPad *New() { return new vtkImageConstantPad; }
};
