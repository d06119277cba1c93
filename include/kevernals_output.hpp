// kevernals_output.hpp -- output and post-processing for the drop-in: TIFF
// writers, the 16-bit rescale and the histogram tools of the reference, on
// top of kevernals_tomo.hpp (no VTK).
//
//   WriteTIFF (16-bit)      as the float32 WriteTIFF of kevernals_tomo.hpp
//                           (the vtkTIFFWriter dumps of recons::ART / MLEM's
//                           verbose mode, Reconstructors.h:47-131, and of the
//                           mains): uncompressed, one page per z slice, rows
//                           written top first (VTK's row 0 is the bottom)
//   RescaleToUInt16         vtkImageShiftScale(scale = (65535 - 1) / max,
//                           unsigned short, clamp on) of the reference's
//                           tomosynthesis reconstructor
//                           (backup/reconstruction/TomosynthesisFBPReconstructor.cpp:57-66)
//   GetHist16Bit, HistMatching16Bit, HistUniformization16Bit, HistHalfTop16Bit
//                           source/commons/HistogramMatchingTools.h:12-179
#pragma once

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "kevernals_tomo.hpp"

// A 16-bit image, x fastest, the unsigned-short vtkImageData of the
// reference's post-processing.
struct ImageU16 {
    int dims[3] = {0, 0, 0};
    std::vector<uint16_t> data;
    size_t size() const { return (size_t)dims[0] * dims[1] * dims[2]; }
};
using ImageU16Ptr = std::shared_ptr<ImageU16>;

// out = clamp((x + 0) * (65535 - 1) / max(x), 0, 65535), truncated to
// unsigned short (vtkImageShiftScale without rounding); max(x) is the
// volume's largest finite value.  A volume whose maximum is not positive
// gives zeros; NaN voxels give 0 and +inf voxels 65535.
inline ImageU16Ptr RescaleToUInt16(const ImageDataPtr &in) {
    auto out = std::make_shared<ImageU16>();
    const int *d = in->GetDimensions();
    for (int i = 0; i < 3; ++i) out->dims[i] = d[i];
    out->data.assign(in->size(), 0);
    double mx = -HUGE_VAL;
    for (size_t i = 0; i < in->size(); ++i)
        if (std::isfinite(in->data()[i])) mx = std::max(mx, (double)in->data()[i]);
    if (!(mx > 0.0)) return out;
    const double scale = (double)(USHRT_MAX - 1) / mx;
    for (size_t i = 0; i < in->size(); ++i) {
        const double v = (double)in->data()[i] * scale;
        out->data[i] = v > 0.0 ? (uint16_t)std::min(v, (double)USHRT_MAX) : (uint16_t)0;   // NaN -> 0
    }
    return out;
}

inline std::vector<int> GetHist16Bit(const ImageU16Ptr &img) {
    std::vector<int> h(1 << 16, 0);
    if (img == nullptr) return h;
    for (uint16_t v : img->data) ++h[v];
    return h;
}

// Maps the image's grey levels so that its cumulative histogram follows the
// expected one (HistogramMatchingTools.h:43-158): the 0 bins of both
// histograms are ignored (the reference treats 0 as a mask), each level takes
// the expected level whose normalised cumulative count is closest, and an
// image whose expected histogram sits on one level of width x height counts
// becomes uniform at that level (the reference compares with one slice's
// pixel count).
inline void HistMatching16Bit(std::vector<int> expected, const ImageU16Ptr &img) {
    if (img == nullptr) return;
    auto original = GetHist16Bit(img);
    const int n = (int)original.size();
    if ((int)expected.size() != n) return;
    int first = 0;
    while (first < n && expected[first] == 0) ++first;
    if (first < n && expected[first] == img->dims[0] * img->dims[1]) {
        std::fill(img->data.begin(), img->data.end(), (uint16_t)first);
        return;
    }
    expected[0] = 0;
    original[0] = 0;
    std::vector<double> ce(n), co(n);
    ce[0] = expected[0];
    co[0] = original[0];
    for (int g = 1; g < n; ++g) {
        ce[g] = ce[g - 1] + expected[g];
        co[g] = co[g - 1] + original[g];
    }
    const double te = ce[n - 1], to = co[n - 1];
    for (int g = 0; g < n; ++g) {
        ce[g] /= te;
        co[g] /= to;
    }
    std::vector<uint16_t> lut(n, 0);
    for (int g = 0; g < n; ++g) {
        const double a = co[g];
        auto up = std::upper_bound(ce.begin(), ce.end(), a);
        int level;
        if (up == ce.end()) level = g;
        else if (up != ce.begin() && a - *(up - 1) < *up - a) level = (int)(up - 1 - ce.begin());
        else level = (int)(up - ce.begin());
        lut[g] = (uint16_t)std::min(std::max(level, 0), (int)USHRT_MAX);
    }
    for (auto &v : img->data) v = lut[v];
}

inline void HistUniformization16Bit(const ImageU16Ptr &img) { HistMatching16Bit(std::vector<int>(1 << 16, 1), img); }

inline void HistHalfTop16Bit(const ImageU16Ptr &img) {
    std::vector<int> h(1 << 16, 1);
    for (int g = 0; g < 1000; ++g) h[g] *= 20;
    HistMatching16Bit(h, img);
}

// 16-bit image to a multi-page TIFF.
inline bool WriteTIFF(const std::string &path, const ImageU16Ptr &img) {
    return kvtomo_detail::write_tiff_pages(path, img->dims[0], img->dims[1], img->dims[2], 2, 1,
                                           reinterpret_cast<const uint8_t *>(img->data.data()));
}
