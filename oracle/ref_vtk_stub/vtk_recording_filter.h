// Stand-ins for the VTK filters that the reference's shift-and-add
// (Reconstructors.h:263-379) assembles (TEST INFRASTRUCTURE).  They compute
// no image: every call is accepted, each GetOutput() is a new empty image
// (heap-allocated: the caller's smart pointer may take it over), and
// vtkExtractVOI::SetVOI records the first row of each extracted projection
// (the projection's first row plus the integer shift the reference computed
// for that slice and view), so the shift rule of the reference's own code can
// be read back (vtk_recorded_shifts, in call order: slice-major, views
// inside).  The ART / MLEM drivers call none of them.
#pragma once

#include <vector>

#include "vtkImageData.h"

inline std::vector<int> vtk_recorded_shifts;

struct vtkRecordingPort {};

class vtkRecordingFilter {
public:
    template <typename... A> void SetInputData(A...) {}
    template <typename... A> void SetInputConnection(A...) {}
    template <typename... A> void AddInputConnection(A...) {}
    vtkRecordingPort *GetOutputPort() { return &m_port; }
    vtkImageData *GetOutput() { return new vtkImageData; }
    void Update() {}
    void UpdateWholeExtent() {}
    template <typename... A> void SetOutputWholeExtent(A...) {}
    template <typename... A> void SetTranslation(A...) {}
    template <typename... A> void SetWeight(A...) {}
    template <typename... A> void SetAppendAxis(A...) {}
    template <typename... A> void SetConstant(A...) {}
    template <typename... A> void SetFileName(A...) {}
    void Write() {}

private:
    vtkRecordingPort m_port;
};
