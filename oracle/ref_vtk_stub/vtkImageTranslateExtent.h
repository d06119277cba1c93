// Stand-in for VTK's vtkImageTranslateExtent (TEST INFRASTRUCTURE), see vtk_recording_filter.h.
#pragma once

#include "vtk_recording_filter.h"

class vtkImageTranslateExtent : public vtkRecordingFilter {
public:
    static vtkImageTranslateExtent *New() { return new vtkImageTranslateExtent; }
};
