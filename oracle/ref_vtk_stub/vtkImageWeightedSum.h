// Stand-in for VTK's vtkImageWeightedSum (TEST INFRASTRUCTURE), see vtk_recording_filter.h.
#pragma once

#include "vtk_recording_filter.h"

class vtkImageWeightedSum : public vtkRecordingFilter {
public:
    static vtkImageWeightedSum *New() { return new vtkImageWeightedSum; }
};
