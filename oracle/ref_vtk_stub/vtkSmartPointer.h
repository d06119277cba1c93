// Minimal stand-in for VTK's vtkSmartPointer (TEST INFRASTRUCTURE, beside
// the vtkImageData stand-in): shared ownership, ->, conversion to the raw
// pointer, comparison with nullptr.
#pragma once

#include <memory>

template <typename T>
class vtkSmartPointer {
public:
    vtkSmartPointer() = default;
    vtkSmartPointer(T *p) : m_p(p) {}
    static vtkSmartPointer New() { return vtkSmartPointer(T::New()); }
    T *operator->() const { return m_p.get(); }
    T *Get() const { return m_p.get(); }
    operator T *() const { return m_p.get(); }
    friend bool operator==(const vtkSmartPointer &a, std::nullptr_t) { return a.m_p == nullptr; }
    friend bool operator!=(const vtkSmartPointer &a, std::nullptr_t) { return a.m_p != nullptr; }

private:
    std::shared_ptr<T> m_p;
};
