// Stand-in for VTK's vtkExtractVOI (TEST INFRASTRUCTURE), see
// vtk_recording_filter.h: SetVOI records the extracted rows' first index.
#pragma once

#include "vtk_recording_filter.h"

class vtkExtractVOI : public vtkRecordingFilter {
public:
    static vtkExtractVOI *New() { return new vtkExtractVOI; }
    void SetVOI(int, int, int y0, int, int, int) { vtk_recorded_shifts.push_back(y0); }
};
