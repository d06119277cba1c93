// kevernals_dicom.hpp -- projection ingestion for the drop-in: a DICOM
// directory reader and the reference's projection preprocessing, on top of
// kevernals_tomo.hpp.
//
//   DICOMReader             source/modules/dataHandling/DICOMReader.h:9-28,
//                           DICOMReader.cpp:16-203
//   DICOMReaderErrorCode    source/modules/dataHandling/DICOMReaderErrorCode.h:19-22
//   LogarithmicScale        the vtkImageCast + vtkImageLogarithmicScale(1)
//                           steps of source/mains/mainReconstruct.cpp:113-124
//
// The reference reads DICOM through vtk-dicom's vtkDICOMReader; this header
// carries a small reader of its own for the files a projection series uses:
// Part-10 files (or bare datasets) in Explicit or Implicit VR Little Endian,
// one frame of 8/16/32-bit integer samples, one sample per pixel.  Other
// transfer syntaxes (big endian, deflated, compressed pixel data) are
// refused with an error.  Conventions taken from vtkDICOMReader's defaults:
// rows are stored bottom-up (memory row 0 is the image's last row) and no
// rescale slope / intercept is applied.  As in the reference, the
// acquisition time is only read from files that carry a PatientID
// (DICOMReader.cpp:121-125); images are ordered by that time as a string,
// the listed indices are removed, and every image is cropped to the
// geometry's detector ROI (bottom-left pixel and size).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <string>
#include <system_error>
#include <vector>

#include "kevernals_tomo.hpp"

enum class DICOMReaderErrorCode { DataFileReadingProblem };

namespace kvtomo_detail {
class DICOMReaderCategory : public std::error_category {
public:
    const char *name() const noexcept override { return "DICOMReaderError"; }
    std::string message(int) const override { return "DICOM file reading failed"; }
};
inline const std::error_category &dicom_reader_category() {
    static DICOMReaderCategory c;
    return c;
}
}  // namespace kvtomo_detail

namespace std {
template <> struct is_error_code_enum<DICOMReaderErrorCode> : public true_type {};
}  // namespace std

inline std::error_code make_error_code(DICOMReaderErrorCode e) {
    return {static_cast<int>(e), kvtomo_detail::dicom_reader_category()};
}

namespace kvdicom {

// One decoded image: samples as float, rows in file order (top row first).
struct Image {
    int rows = 0, cols = 0;
    bool has_patient_id = false;
    std::string acquisition_time;
    std::vector<float> pixels;
};

class Parser {
public:
    Parser(const std::vector<uint8_t> &b) : b_(b) {}

    bool parse(Image &img, std::string &err) {
        size_t pos = 0;
        if (b_.size() >= 132 && std::memcmp(&b_[128], "DICM", 4) == 0) pos = 132;
        bool explicit_vr = pos != 0;    // a bare dataset without meta header: Implicit VR Little Endian
        // file meta information: always Explicit VR Little Endian
        std::string ts;
        while (pos + 8 <= b_.size() && u16(pos) == 0x0002) {
            Elem e;
            if (!element(pos, true, e, err)) return false;
            if (e.tag == 0x00020010) ts = text(e);
            pos = e.next;
        }
        if (!ts.empty()) {
            if (ts == "1.2.840.10008.1.2") explicit_vr = false;
            else if (ts == "1.2.840.10008.1.2.1") explicit_vr = true;
            else {
                err = "unsupported transfer syntax " + kvtomo_detail::printable(ts);
                return false;
            }
        }
        int bits = 0, pixrep = 0, spp = 1, frames = 1;
        const Elem *pixel = nullptr;
        Elem pix;
        while (pos + 8 <= b_.size()) {
            Elem e;
            if (!element(pos, explicit_vr, e, err)) return false;
            switch (e.tag) {
            case 0x00100020: img.has_patient_id = true; break;
            case 0x00080032: img.acquisition_time = text(e); break;
            case 0x00280002: spp = num(e); break;
            case 0x00280008: frames = std::atoi(text(e).c_str()); break;
            case 0x00280010: img.rows = num(e); break;
            case 0x00280011: img.cols = num(e); break;
            case 0x00280100: bits = num(e); break;
            case 0x00280103: pixrep = num(e); break;
            case 0x7FE00010: pix = e; pixel = &pix; break;
            default: break;
            }
            pos = e.next;
            if (pixel) break;
        }
        if (pixel == nullptr) { err = "no pixel data"; return false; }
        if (pixel->undefined) { err = "encapsulated (compressed) pixel data is not supported"; return false; }
        if (spp != 1 || frames > 1) { err = "only single-frame, single-sample images are supported"; return false; }
        if (img.rows <= 0 || img.cols <= 0) { err = "missing image size"; return false; }
        if (bits != 8 && bits != 16 && bits != 32) { err = "unsupported bits allocated " + std::to_string(bits); return false; }
        const size_t n = (size_t)img.rows * img.cols, bytes = n * (bits / 8);
        if (pixel->len < bytes || pixel->val + bytes > b_.size()) { err = "truncated pixel data"; return false; }
        img.pixels.resize(n);
        const uint8_t *p = &b_[pixel->val];
        for (size_t i = 0; i < n; ++i) {
            if (bits == 8) img.pixels[i] = pixrep ? (float)(int8_t)p[i] : (float)p[i];
            else if (bits == 16) {
                const uint16_t v = (uint16_t)(p[2 * i] | (p[2 * i + 1] << 8));
                img.pixels[i] = pixrep ? (float)(int16_t)v : (float)v;
            } else {
                const uint32_t v = (uint32_t)p[4 * i] | ((uint32_t)p[4 * i + 1] << 8) |
                                   ((uint32_t)p[4 * i + 2] << 16) | ((uint32_t)p[4 * i + 3] << 24);
                img.pixels[i] = pixrep ? (float)(int32_t)v : (float)v;
            }
        }
        return true;
    }

private:
    struct Elem {
        uint32_t tag = 0;
        size_t val = 0, len = 0, next = 0;
        bool undefined = false;
        char vr[2] = {0, 0};
    };
    const std::vector<uint8_t> &b_;

    uint16_t u16(size_t p) const { return (uint16_t)(b_[p] | (b_[p + 1] << 8)); }
    uint32_t u32(size_t p) const {
        return (uint32_t)b_[p] | ((uint32_t)b_[p + 1] << 8) | ((uint32_t)b_[p + 2] << 16) | ((uint32_t)b_[p + 3] << 24);
    }
    static bool long_vr(const char *vr) {
        static const char *l[] = {"OB", "OD", "OF", "OL", "OV", "OW", "SQ", "SV", "UC", "UN", "UR", "UT", "UV"};
        for (const char *x : l)
            if (vr[0] == x[0] && vr[1] == x[1]) return true;
        return false;
    }
    std::string text(const Elem &e) const {
        std::string s(reinterpret_cast<const char *>(&b_[e.val]), e.len);
        while (!s.empty() && (s.back() == ' ' || s.back() == '\0')) s.pop_back();
        size_t a = 0;
        while (a < s.size() && s[a] == ' ') ++a;
        return s.substr(a);
    }
    int num(const Elem &e) const {
        if (e.len >= 4 && (e.vr[0] == 'U' && e.vr[1] == 'L')) return (int)u32(e.val);
        if (e.len >= 2) return (int)u16(e.val);
        return 0;
    }
    // One data element at pos; undefined-length sequences and items are
    // walked to their delimiters so `next` lands after them.
    bool element(size_t pos, bool explicit_vr, Elem &e, std::string &err) const {
        if (pos + 8 > b_.size()) { err = "truncated element header"; return false; }
        e.tag = ((uint32_t)u16(pos) << 16) | u16(pos + 2);
        size_t p = pos + 4;
        uint32_t len;
        const bool item_tag = (e.tag >> 16) == 0xFFFE;
        if (explicit_vr && !item_tag) {
            e.vr[0] = (char)b_[p];
            e.vr[1] = (char)b_[p + 1];
            if (long_vr(e.vr)) {
                if (p + 8 > b_.size()) { err = "truncated element header"; return false; }
                len = u32(p + 4);
                p += 8;
            } else {
                len = u16(p + 2);
                p += 4;
            }
        } else {
            len = u32(p);
            p += 4;
        }
        e.val = p;
        if (len != 0xFFFFFFFFu) {
            e.len = len;
            e.next = p + len;
            if (e.next > b_.size()) { err = "element runs past the end of the file"; return false; }
            return true;
        }
        // undefined length: a sequence, an item, or encapsulated pixel data
        e.undefined = true;
        const uint32_t end_tag = e.tag == 0xFFFEE000u ? 0xFFFEE00Du : 0xFFFEE0DDu;
        const bool nested_explicit = explicit_vr && e.tag != 0x7FE00010u;
        size_t q = p;
        for (;;) {
            if (q + 8 > b_.size()) { err = "unterminated sequence"; return false; }
            const uint32_t t = ((uint32_t)u16(q) << 16) | u16(q + 2);
            if (t == end_tag) {
                e.len = q - p;
                e.next = q + 8;
                return true;
            }
            Elem c;
            if (!element(q, nested_explicit, c, err)) return false;
            q = c.next;
        }
    }
};

inline bool read_file(const std::string &path, Image &img, std::string &err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    std::vector<uint8_t> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    return Parser(b).parse(img, err);
}

}  // namespace kvdicom

class DICOMReader {
public:
    DICOMReader() = delete;
    DICOMReader(TomoGeometry *p_tomoGeometry) : m_geo(p_tomoGeometry) {}

    // One projection image, cropped to the geometry's detector ROI.
    Result<ImageDataPtr> Read(const std::string &p_dicomFilePath) const {
        kvdicom::Image img;
        if (!kvdicom::read_file(p_dicomFilePath, img, m_error)) return make_error_code(DICOMReaderErrorCode::DataFileReadingProblem);
        auto out = ImageData::New();
        if (!crop_into(img, out, 1, 0)) return make_error_code(DICOMReaderErrorCode::DataFileReadingProblem);
        return out;
    }

    // Every .dcm / .DCM file of a directory, ordered by acquisition time,
    // without the listed positions (indices into the ordered list), cropped
    // to the ROI and stacked along z (one slice per view).
    Result<ImageDataPtr> ReadDirectory(const std::string &p_dir, const std::vector<int> &p_indicesToRemove) const {
        namespace fs = std::filesystem;
        std::error_code ec;
        if (!fs::exists(p_dir, ec)) {
            m_error = "directory does not exist: " + p_dir;
            return make_error_code(DICOMReaderErrorCode::DataFileReadingProblem);
        }
        struct Entry {
            kvdicom::Image img;
            std::string time, name;
        };
        std::vector<Entry> images;
        for (const auto &de : fs::directory_iterator(p_dir, ec)) {
            const auto ext = de.path().extension().generic_string();
            if (ext != ".dcm" && ext != ".DCM") continue;
            Entry e;
            e.name = de.path().generic_string();
            if (!kvdicom::read_file(e.name, e.img, m_error)) {
                m_error = e.name + ": " + m_error;
                return make_error_code(DICOMReaderErrorCode::DataFileReadingProblem);
            }
            if (e.img.has_patient_id) e.time = e.img.acquisition_time;
            images.push_back(std::move(e));
        }
        std::stable_sort(images.begin(), images.end(),
                         [](const Entry &a, const Entry &b) { return a.time < b.time; });
        auto idx = p_indicesToRemove;
        std::sort(idx.begin(), idx.end(), std::greater<int>());
        for (int i : idx) {
            if (i < 0 || i >= (int)images.size()) {
                m_error = "index to remove out of range: " + std::to_string(i);
                return make_error_code(DICOMReaderErrorCode::DataFileReadingProblem);
            }
            images.erase(images.begin() + i);
        }
        if (images.empty()) {
            m_error = "no DICOM image in " + p_dir;
            return make_error_code(DICOMReaderErrorCode::DataFileReadingProblem);
        }
        auto out = ImageData::New();
        for (size_t k = 0; k < images.size(); ++k)
            if (!crop_into(images[k].img, out, (int)images.size(), (int)k))
                return make_error_code(DICOMReaderErrorCode::DataFileReadingProblem);
        return out;
    }

    // Why the last call failed.
    const std::string &LastError() const { return m_error; }

private:
    // Copies the ROI of img (rows bottom-up) into slice k of out.
    bool crop_into(const kvdicom::Image &img, const ImageDataPtr &out, int nslices, int k) const {
        const Size2D bl = m_geo->GetProjectionROIsBLPixelPositionOnDetector();
        const Size2D sz = m_geo->projectionsRoisSize();
        if (bl.x < 0 || bl.y < 0 || sz.x <= 0 || sz.y <= 0 || bl.x + sz.x > img.cols || bl.y + sz.y > img.rows) {
            m_error = "the detector ROI does not fit the " + std::to_string(img.cols) + " x " +
                      std::to_string(img.rows) + " image";
            return false;
        }
        if (k == 0) {
            out->SetDimensions(sz.x, sz.y, nslices);
            out->AllocateScalars();
        }
        float *dst = out->data() + (size_t)k * sz.x * sz.y;
        for (int y = 0; y < sz.y; ++y) {
            const int file_row = img.rows - 1 - (bl.y + y);    // bottom-up memory rows
            const float *src = img.pixels.data() + (size_t)file_row * img.cols + bl.x;
            std::copy(src, src + sz.x, dst + (size_t)y * sz.x);
        }
        return true;
    }

    TomoGeometry *m_geo;
    mutable std::string m_error;
};

// The reference's projection preprocessing: cast to float (the reader's
// output already is) and c * log(1 + x), with -c * log(1 - x) for negative
// samples (vtkImageLogarithmicScale, computed in double).
inline ImageDataPtr LogarithmicScale(const ImageDataPtr &in, double c = 1.0) {
    auto out = ImageData::New();
    const int *d = in->GetDimensions();
    out->SetDimensions(d[0], d[1], d[2]);
    double sp[3], org[3];
    in->GetSpacing(sp);
    in->GetOrigin(org);
    out->SetSpacing(sp[0], sp[1], sp[2]);
    out->SetOrigin(org[0], org[1], org[2]);
    out->AllocateScalars();
    const float *s = in->data();
    float *o = out->data();
    for (size_t i = 0; i < in->size(); ++i) {
        const double x = s[i];
        o[i] = (float)(x > 0.0 ? c * std::log(x + 1.0) : -c * std::log(1.0 - x));
    }
    return out;
}
