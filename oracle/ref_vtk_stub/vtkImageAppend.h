// Stand-in for VTK's vtkImageAppend (TEST INFRASTRUCTURE), see vtk_recording_filter.h.
#pragma once

#include "vtk_recording_filter.h"

class vtkImageAppend : public vtkRecordingFilter {
public:
    static vtkImageAppend *New() { return new vtkImageAppend; }
};
