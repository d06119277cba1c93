// Stand-in for VTK's vtkTIFFWriter (TEST INFRASTRUCTURE), see vtk_recording_filter.h.
#pragma once

#include "vtk_recording_filter.h"

class vtkTIFFWriter : public vtkRecordingFilter {
public:
    static vtkTIFFWriter *New() { return new vtkTIFFWriter; }
};
