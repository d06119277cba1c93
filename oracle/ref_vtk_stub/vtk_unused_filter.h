// Compile-only stand-ins for the VTK filters that the reference's
// shift-and-add (Reconstructors.h:263-379) assembles (TEST INFRASTRUCTURE).
// The driver checker runs the reference's ART and MLEM only; a call into any
// of these ends the process, so no result can silently depend on them.
#pragma once

#include <cstdio>
#include <cstdlib>

#include "vtkImageData.h"

struct vtkUnusedPort {};

class vtkUnusedFilter {
public:
    [[noreturn]] static void unused() {
        std::fprintf(stderr, "reference checker: a VTK filter stand-in was called\n");
        std::abort();
    }
    template <typename... A> void SetInputData(A...) { unused(); }
    template <typename... A> void SetInputConnection(A...) { unused(); }
    template <typename... A> void AddInputConnection(A...) { unused(); }
    vtkUnusedPort *GetOutputPort() { unused(); }
    vtkImageData *GetOutput() { unused(); }
    void Update() { unused(); }
    void UpdateWholeExtent() { unused(); }
    template <typename... A> void SetOutputWholeExtent(A...) { unused(); }
    template <typename... A> void SetVOI(A...) { unused(); }
    template <typename... A> void SetTranslation(A...) { unused(); }
    template <typename... A> void SetWeight(A...) { unused(); }
    template <typename... A> void SetAppendAxis(A...) { unused(); }
    template <typename... A> void SetConstant(A...) { unused(); }
    template <typename... A> void SetFileName(A...) { unused(); }
    void Write() { unused(); }
};
