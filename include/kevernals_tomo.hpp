// kevernals_tomo.hpp -- C++ drop-in for the Kevernals projection /
// reconstruction modules, over the kvtomo C ABI (kvtomo.h).
//
// Same names, argument meaning and error behaviour as the reference:
//   Projector               source/modules/reconstruction/Projector.h:10-28
//   recons::ART / MLEM / BackProjection / ShiftAndAdd
//                           source/modules/reconstruction/Reconstructors.h:19-379
//   ReconstructorsErrorCode source/modules/reconstruction/ReconstructorsErrorCode.h:19-26
//   Result<T>               source/commons/Result.h:17-41 (value or std::error_code)
//   TomoGeometry accessors  source/modules/geometry/TomoGeometry.h:34-89
// Differences, by design:
//   * ImageDataPtr is a small reference-counted headless image (dimensions,
//     spacing, origin, float32 buffer) instead of vtkSmartPointer<vtkImageData>.
//   * TomoGeometry is built from values, or read from the reference's XML
//     geometry files (TomoGeometry(path), source/modules/geometry/
//     TomoGeometry.cpp:13-434) by a small XML reader of this header; it keeps
//     the reference's conventions: volume-centred frame, common source x/z
//     and detector z, one ROI size and pixel spacing.  An unreadable file
//     gives an invalid geometry (IsValid() false, ErrorMessage() says why)
//     instead of the reference's console message.
//   * Projector takes an operator family: KV_FAMILY_RC (default) reproduces
//     the reference kernels; KV_FAMILY_EXACT is the Siddon line integral and
//     its exact transpose.
//   * Errors never exit the process: CUDA failures surface as error codes.
//   * All functions are inline (the reference defines them in a header
//     without `inline`).
#pragma once

#include <algorithm>
#include <cctype>
#include <functional>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <limits>
#include <sstream>
#include <memory>
#include <optional>
#include <ostream>
#include <stdexcept>
#include <string>
#include <system_error>
#include <vector>

#include "kvtomo.h"

// ---------------------------------------------------------------- values

struct Position2D {
    float x = 0.f, y = 0.f;
};
struct Position3D {
    float x = 0.f, y = 0.f, z = 0.f;
};
struct Size2D {
    int x = 0, y = 0;
};
struct Size3D {
    int x = 0, y = 0, z = 0;
};
struct PixelSpacing {
    float x = 0.f, y = 0.f;
};
struct VoxelSpacing {
    float x = 0.f, y = 0.f, z = 0.f;
};
using WSize3D = Position3D;
using WSize2D = Position2D;

// ---------------------------------------------------------------- errors

enum class ReconstructorsErrorCode { ART = 1, BackProjectionFailed, ProjectionFailed, MLEM, ShiftAndAdd };

namespace kvtomo_detail {
class ReconstructorsCategory : public std::error_category {
public:
    const char *name() const noexcept override { return "Reconstructors"; }
    std::string message(int c) const override {
        switch (static_cast<ReconstructorsErrorCode>(c)) {
        case ReconstructorsErrorCode::ART: return "ART reconstruction failed";
        case ReconstructorsErrorCode::BackProjectionFailed: return "back projection failed";
        case ReconstructorsErrorCode::ProjectionFailed: return "projection failed";
        case ReconstructorsErrorCode::MLEM: return "MLEM reconstruction failed";
        case ReconstructorsErrorCode::ShiftAndAdd: return "shift and add failed";
        }
        return "unknown reconstructors error";
    }
};
inline const std::error_category &reconstructors_category() {
    static ReconstructorsCategory c;
    return c;
}

// n positions from `first` by repeated float addition of `step`
inline std::vector<float> axis_positions(float first, float step, int n) {
    std::vector<float> v(n > 0 ? n : 0);
    if (n > 0) v[0] = first;
    for (int i = 1; i < n; ++i) v[i] = v[i - 1] + step;
    return v;
}
// per view: positions along x (or y) of its n pixels from the view's corner
inline std::vector<std::vector<float>> view_positions(const std::vector<Position2D> &corners, bool x, float step,
                                                      int n) {
    std::vector<std::vector<float>> out;
    for (const auto &c : corners) out.push_back(axis_positions(x ? c.x : c.y, step, n));
    return out;
}
// every pixel of every view, views then rows then columns
inline std::vector<Position2D> pixel_positions(const std::vector<std::vector<float>> &xs,
                                               const std::vector<std::vector<float>> &ys) {
    std::vector<Position2D> out;
    for (size_t p = 0; p < xs.size(); ++p)
        for (float y : ys[p])
            for (float x : xs[p]) out.push_back({x, y});
    return out;
}
inline std::vector<int> indices(size_t n) {
    std::vector<int> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = static_cast<int>(i);
    return v;
}

// A value read from a file, fit for an error message: printable ASCII only
// (anything else becomes '?'), at most 64 characters.
inline std::string printable(const std::string &v) {
    std::string out;
    for (size_t i = 0; i < v.size() && i < 64; ++i) {
        const unsigned char c = static_cast<unsigned char>(v[i]);
        out += (c >= 0x20 && c < 0x7F) ? static_cast<char>(c) : '?';
    }
    return out;
}
}  // namespace kvtomo_detail

namespace std {
template <> struct is_error_code_enum<ReconstructorsErrorCode> : public true_type {};
}  // namespace std

inline std::error_code make_error_code(ReconstructorsErrorCode e) {
    return {static_cast<int>(e), kvtomo_detail::reconstructors_category()};
}

// commons/PrintErrorCode.h: "<category>:<value> <message>. Details: <comment>"
inline std::string PrintErrorCode(const std::error_code &p_errorCode,
                                  const std::string &p_additionalComment = std::string("none.")) {
    std::stringstream stream;
    stream << p_errorCode << " " << p_errorCode.message() << ". Details: " << p_additionalComment;
    return stream.str();
}

// Value-or-error, the subset of outcome::result the reference uses.
// The error state is kept apart from the code's value: an enumerator whose
// value is 0 (DICOMReaderErrorCode::DataFileReadingProblem) is still an
// error, as in outcome::result.
template <typename T> class Result {
public:
    Result(T v) : m_value(std::move(v)) {}
    Result(std::error_code e) : m_error(e), m_failed(true) {}
    Result(ReconstructorsErrorCode e) : m_error(make_error_code(e)), m_failed(true) {}
    bool has_value() const { return !m_failed; }
    bool has_error() const { return m_failed; }
    explicit operator bool() const { return has_value(); }
    const T &value() const {
        if (m_failed) throw std::system_error(m_error);
        return m_value;
    }
    T &value() {
        if (m_failed) throw std::system_error(m_error);
        return m_value;
    }
    std::error_code error() const { return m_error; }

private:
    T m_value{};
    std::error_code m_error{};
    bool m_failed = false;
};

// ---------------------------------------------------------------- images

class ImageData {
public:
    static std::shared_ptr<ImageData> New() { return std::make_shared<ImageData>(); }
    void SetDimensions(int x, int y, int z) {
        m_dims[0] = x;
        m_dims[1] = y;
        m_dims[2] = z;
    }
    int *GetDimensions() { return m_dims; }
    const int *GetDimensions() const { return m_dims; }
    void SetSpacing(double x, double y, double z) {
        m_spacing[0] = x;
        m_spacing[1] = y;
        m_spacing[2] = z;
    }
    void GetSpacing(double out[3]) const {
        for (int i = 0; i < 3; ++i) out[i] = m_spacing[i];
    }
    const double *GetSpacing() const { return m_spacing; }
    void SetOrigin(double x, double y, double z) {
        m_origin[0] = x;
        m_origin[1] = y;
        m_origin[2] = z;
    }
    void GetOrigin(double out[3]) const {
        for (int i = 0; i < 3; ++i) out[i] = m_origin[i];
    }
    const double *GetOrigin() const { return m_origin; }
    // whole extent [0, nx-1, 0, ny-1, 0, nz-1], as vtkImageData::GetExtent
    void GetExtent(int out[6]) const {
        for (int i = 0; i < 3; ++i) {
            out[2 * i] = 0;
            out[2 * i + 1] = m_dims[i] - 1;
        }
    }
    long long GetNumberOfPoints() const { return static_cast<long long>(size()); }
    // dimensions, spacing, origin and a copy of the scalars
    void DeepCopy(const ImageData *src) {
        if (src == nullptr || src == this) return;
        *this = *src;
    }
    void DeepCopy(const std::shared_ptr<ImageData> &src) { DeepCopy(src.get()); }
    // VTK_FLOAT with one component is the only scalar type used on this path.
    void AllocateScalars(int = 0, int = 1) { m_data.assign(size(), 0.f); }
    void *GetScalarPointer() { return m_data.data(); }
    // the scalar at voxel (x, y, z), x fastest; nullptr outside the image
    void *GetScalarPointer(int x, int y, int z) {
        if (x < 0 || y < 0 || z < 0 || x >= m_dims[0] || y >= m_dims[1] || z >= m_dims[2] || m_data.empty())
            return nullptr;
        return m_data.data() + (static_cast<size_t>(z) * m_dims[1] + y) * m_dims[0] + x;
    }
    // one component (c = 0) per voxel
    float GetScalarComponentAsFloat(int x, int y, int z, int c) {
        const float *p = static_cast<const float *>(GetScalarPointer(x, y, z));
        return (p != nullptr && c == 0) ? *p : 0.f;
    }
    void SetScalarComponentFromFloat(int x, int y, int z, int c, float v) {
        float *p = static_cast<float *>(GetScalarPointer(x, y, z));
        if (p != nullptr && c == 0) *p = v;
    }
    const float *data() const { return m_data.data(); }
    float *data() { return m_data.data(); }
    size_t size() const { return (size_t)m_dims[0] * m_dims[1] * m_dims[2]; }

private:
    int m_dims[3] = {0, 0, 0};
    double m_spacing[3] = {1, 1, 1};
    double m_origin[3] = {0, 0, 0};
    std::vector<float> m_data;
};
using ImageDataPtr = std::shared_ptr<ImageData>;

// ---------------------------------------------------------------- geometry

// ---------------------------------------------------------------- XML

namespace kvxml {

// A minimal XML element tree: element names, concatenated character data,
// child elements.  Enough for the geometry files (no namespaces, DTDs or
// processing of attributes, which those files do not use).
struct Node {
    std::string name, text;
    std::vector<Node> children;
    const Node *child(const std::string &n) const {
        for (const auto &c : children)
            if (c.name == n) return &c;
        return nullptr;
    }
};

class Parser {
public:
    explicit Parser(const std::string &src) : s_(src) {}
    bool parse(Node &root, std::string &err) {
        skip_misc();
        return element(root, err);
    }

private:
    const std::string &s_;
    size_t i_ = 0;
    bool starts(const char *t) const { return s_.compare(i_, std::char_traits<char>::length(t), t) == 0; }
    void skip_ws() {
        while (i_ < s_.size() && std::isspace(static_cast<unsigned char>(s_[i_]))) ++i_;
    }
    bool skip_past(const char *t) {
        const size_t k = s_.find(t, i_);
        if (k == std::string::npos) return false;
        i_ = k + std::char_traits<char>::length(t);
        return true;
    }
    // declarations, comments, doctype before the root element
    void skip_misc() {
        for (;;) {
            skip_ws();
            if (starts("<?")) { if (!skip_past("?>")) return; }
            else if (starts("<!--")) { if (!skip_past("-->")) return; }
            else if (starts("<!")) { if (!skip_past(">")) return; }
            else return;
        }
    }
    // the five predefined entities, in one left-to-right pass (so "&amp;lt;"
    // gives "&lt;"); anything else is kept as written
    static void decode(std::string &t) {
        static const std::pair<const char *, char> ents[] = {
            {"&lt;", '<'}, {"&gt;", '>'}, {"&quot;", '"'}, {"&apos;", '\''}, {"&amp;", '&'}};
        std::string out;
        out.reserve(t.size());
        for (size_t i = 0; i < t.size();) {
            bool hit = false;
            if (t[i] == '&') {
                for (const auto &e : ents) {
                    const size_t n = std::char_traits<char>::length(e.first);
                    if (t.compare(i, n, e.first) == 0) {
                        out += e.second;
                        i += n;
                        hit = true;
                        break;
                    }
                }
            }
            if (!hit) out += t[i++];
        }
        t.swap(out);
    }
    // nesting deeper than this is refused (the geometry schema uses four levels)
    static constexpr int kMaxDepth = 64;
    bool element(Node &n, std::string &err, int depth = 0) {
        if (depth > kMaxDepth) { err = "elements nested too deeply"; return false; }
        if (!starts("<")) { err = "expected an element"; return false; }
        ++i_;
        const size_t b = i_;
        while (i_ < s_.size() && !std::isspace(static_cast<unsigned char>(s_[i_])) && s_[i_] != '>' && s_[i_] != '/')
            ++i_;
        n.name = s_.substr(b, i_ - b);
        const size_t close = s_.find('>', i_);
        if (close == std::string::npos) { err = "unterminated tag <" + n.name; return false; }
        const bool empty = close > 0 && s_[close - 1] == '/';
        i_ = close + 1;
        if (empty) return true;
        for (;;) {
            if (i_ >= s_.size()) { err = "missing </" + n.name + ">"; return false; }
            if (starts("<!--")) { if (!skip_past("-->")) { err = "unterminated comment"; return false; } continue; }
            if (starts("<![CDATA[")) {
                const size_t e = s_.find("]]>", i_);
                if (e == std::string::npos) { err = "unterminated CDATA"; return false; }
                n.text += s_.substr(i_ + 9, e - i_ - 9);
                i_ = e + 3;
                continue;
            }
            if (starts("</")) {
                const size_t e = s_.find('>', i_);
                if (e == std::string::npos) { err = "unterminated </" + n.name; return false; }
                i_ = e + 1;
                return true;
            }
            if (starts("<")) {
                n.children.emplace_back();
                if (!element(n.children.back(), err, depth + 1)) return false;
                continue;
            }
            const size_t e = s_.find('<', i_);
            std::string t = s_.substr(i_, (e == std::string::npos ? s_.size() : e) - i_);
            decode(t);
            n.text += t;
            i_ = e == std::string::npos ? s_.size() : e;
        }
    }
};

inline std::vector<std::string> words(const std::string &t) {
    std::istringstream in(t);
    std::vector<std::string> w;
    std::string x;
    while (in >> x) w.push_back(x);
    return w;
}

// "a b c" -> three numbers (the reference's Dim3::FromString: exactly three
// whitespace-separated words, each read with std::stod)
inline bool triple(const Node *n, double (&v)[3]) {
    if (n == nullptr) return false;
    const auto w = words(n->text);
    if (w.size() != 3) return false;
    try {
        for (int k = 0; k < 3; ++k) v[k] = std::stod(w[k]);
    } catch (const std::exception &) {
        return false;
    }
    return true;
}

inline bool number(const Node *n, double &v) {
    if (n == nullptr) return false;
    try {
        v = std::stod(n->text);
    } catch (const std::exception &) {
        return false;
    }
    return true;
}

}  // namespace kvxml

class TomoGeometry;

// Read-only views of a geometry's parts under the reference's class names,
// as TomoGeometry::GetVolume / GetProjections / GetProjectionsRois /
// GetTable return them (TomoGeometry.h:86-89): the value accessors of
// TomoVolume (TomoVolume.h:49-64), TomoProjectionsSet
// (TomoProjectionsSet.h:32-41) and TomoTable (TomoTable.h:16-23), read from
// the owning TomoGeometry when called (so they follow its changes).  The
// reference's setters, point-location helpers and RemoveProjection /
// RemoveSource are not provided: the geometry changes through TomoGeometry.
class TomoVolume {
public:
    explicit TomoVolume(const TomoGeometry *g = nullptr) : m_g(g) {}
    int GetVoxelsNumber() const;
    float GetSize() const;
    Size3D GetSize3D() const;
    WSize3D GetWSize3D() const;
    Position3D GetBottomLeftFront() const;
    Position3D GetTopRightBack() const;
    VoxelSpacing GetVoxelSpacing() const;
    std::vector<float> GetXPositions() const;
    std::vector<float> GetYPositions() const;
    std::vector<float> GetZPositions() const;
    std::vector<Position3D> GetGridPositions() const;
    std::vector<int> GetVoxelsIndices() const;

private:
    const TomoGeometry *m_g;
};

class TomoProjectionsSet {
public:
    explicit TomoProjectionsSet(const TomoGeometry *g = nullptr, bool rois = false) : m_g(g), m_rois(rois) {}
    std::vector<Position2D> GetBottomLeftPositions() const;
    Size2D GetSize() const;
    WSize2D GetWSize() const;
    PixelSpacing GetPixelSpacing() const;
    std::vector<std::vector<float>> GetXPositions() const;
    std::vector<std::vector<float>> GetYPositions() const;
    std::vector<Position2D> GetProjectionPositions() const;
    std::vector<int> GetProjectionPixelsIndices() const;
    int GetNProjections() const;

private:
    const TomoGeometry *m_g;
    bool m_rois;
};

class TomoTable {
public:
    explicit TomoTable(const TomoGeometry *g = nullptr) : m_g(g) {}
    int GetSourcesNumber() const;
    std::vector<float> GetSourcesYPositions() const;
    float GetSourcesXCommonPosition() const;
    float GetSourcesZCommonPosition() const;
    float GetDetectorsZCommonPosition() const;

private:
    const TomoGeometry *m_g;
};

class TomoGeometry {
public:
    // Reads a geometry file of the reference's format (TomoGeometry.cpp:13-434):
    //   Rotation/center                     fulcrum (file frame)
    //   Grid/center, Grid/scale, Grid/resolution   volume centre, voxel
    //                                       spacing and voxel counts, each
    //                                       written z y x
    //   XRay/sources/*                      one source position per view
    //   Camera/totalWidth, totalHeight      detector extent (mm)
    //   Camera/pixelWidth, pixelHeight      detector pixel counts
    //   Camera/references/*                 per-view detector bottom-left corner
    //   Radios/rois/*                       the ROI, "x0 y0 . . x1 y1" pixels,
    //                                       the same for every view
    // Positions are moved to the volume-centred frame (minus Grid/center);
    // the detector plane is the mean detector z (summed in double); the
    // ROI's bottom-left position of view i is the detector corner plus the
    // pixel pitch added pixel by pixel in float (TomoProjectionsSet.cpp:
    // 172-190, 152-155), the pitch being extent / count (PixelSpacing.cpp).
    explicit TomoGeometry(const std::string &xmlPath) : m_filePath(xmlPath) { m_valid = read_xml(xmlPath); }

private:
    bool read_xml(const std::string &xmlPath) {
        std::ifstream f(xmlPath, std::ios::binary);
        if (!f) { m_error = "cannot open " + xmlPath; return false; }
        std::stringstream ss;
        ss << f.rdbuf();
        const std::string src = ss.str();
        kvxml::Node root;
        std::string err;
        if (!kvxml::Parser(src).parse(root, err)) {
            m_error = "XML: " + kvtomo_detail::printable(err);
            return false;
        }
        auto fail = [this](const std::string &m) { m_error = m; return false; };
        // a count as the reference reads it (double -> float -> int), refused
        // when it is not a positive number up to kMaxAxis
        auto count = [](double v, int &out) {
            const float f = static_cast<float>(v);
            if (!(f >= 1.f && f <= static_cast<float>(kMaxAxis))) return false;
            out = static_cast<int>(f);
            return true;
        };
        using kvxml::Node;
        double v[3];
        const Node *rot = root.child("Rotation");
        if (!kvxml::triple(rot ? rot->child("center") : nullptr, v)) return fail("Rotation/center missing or unreadable");
        m_fulcrum = {static_cast<float>(v[0]), static_cast<float>(v[1]), static_cast<float>(v[2])};
        const Node *grid = root.child("Grid");
        if (grid == nullptr) return fail("Grid missing");
        double c[3], sc[3], res[3];
        if (!kvxml::triple(grid->child("center"), c)) return fail("Grid/center missing or unreadable");
        if (!kvxml::triple(grid->child("scale"), sc)) return fail("Grid/scale missing or unreadable");
        if (!kvxml::triple(grid->child("resolution"), res)) return fail("Grid/resolution missing or unreadable");
        const float cx = static_cast<float>(c[0]), cy = static_cast<float>(c[1]), cz = static_cast<float>(c[2]);
        m_spacing = {static_cast<float>(sc[2]), static_cast<float>(sc[1]), static_cast<float>(sc[0])};
        if (!count(res[2], m_size.x) || !count(res[1], m_size.y) || !count(res[0], m_size.z))
            return fail("Grid/resolution must be positive counts up to " + std::to_string(kMaxAxis));
        const Node *xr = root.child("XRay");
        const Node *srcs = xr ? xr->child("sources") : nullptr;
        if (srcs == nullptr || srcs->children.empty()) return fail("XRay/sources missing or empty");
        std::vector<Position3D> sources;
        for (const auto &sn : srcs->children) {
            if (!kvxml::triple(&sn, v)) return fail("an XRay/sources entry is unreadable");
            sources.push_back({static_cast<float>(v[0]) - cx, static_cast<float>(v[1]) - cy,
                               static_cast<float>(v[2]) - cz});
        }
        const Node *cam = root.child("Camera");
        if (cam == nullptr) return fail("Camera missing");
        double tw, th, pw, ph;
        if (!kvxml::number(cam->child("totalWidth"), tw) || static_cast<float>(tw) == 0.f)
            return fail("Camera/totalWidth missing, unreadable or zero");
        if (!kvxml::number(cam->child("totalHeight"), th) || static_cast<float>(th) == 0.f)
            return fail("Camera/totalHeight missing, unreadable or zero");
        if (!kvxml::number(cam->child("pixelWidth"), pw) || static_cast<float>(pw) == 0.f)
            return fail("Camera/pixelWidth missing, unreadable or zero");
        if (!kvxml::number(cam->child("pixelHeight"), ph) || static_cast<float>(ph) == 0.f)
            return fail("Camera/pixelHeight missing, unreadable or zero");
        Size2D det_px{0, 0};
        if (!count(pw, det_px.x) || !count(ph, det_px.y))
            return fail("Camera pixel counts must be positive counts up to " + std::to_string(kMaxAxis));
        m_detWSize = {static_cast<float>(tw), static_cast<float>(th)};
        m_pixel = {m_detWSize.x / static_cast<float>(det_px.x), m_detWSize.y / static_cast<float>(det_px.y)};
        const Node *refs = cam->child("references");
        if (refs == nullptr || refs->children.empty()) return fail("Camera/references missing or empty");
        std::vector<Position2D> det_bl;
        double zsum = 0.0;
        for (const auto &rn : refs->children) {
            if (!kvxml::triple(&rn, v)) return fail("a Camera/references entry is unreadable");
            det_bl.push_back({static_cast<float>(v[0]) - cx, static_cast<float>(v[1]) - cy});
            zsum += static_cast<float>(v[2]) - cz;
        }
        if (det_bl.size() != sources.size()) return fail("one detector reference per source is required");
        m_detZ = static_cast<float>(zsum) / static_cast<float>(det_bl.size());
        const Node *radios = root.child("Radios");
        const Node *rois = radios ? radios->child("rois") : nullptr;
        if (rois == nullptr || rois->children.empty()) return fail("Radios/rois missing or empty");
        int bl[2] = {0, 0}, tr[2] = {0, 0};
        for (size_t k = 0; k < rois->children.size(); ++k) {
            const auto w = kvxml::words(rois->children[k].text);
            if (w.size() < 6) return fail("a Radios/rois entry is unreadable");
            int cur[4];
            try {
                const size_t idx[4] = {0, 1, 4, 5};
                for (int q = 0; q < 4; ++q) {
                    const double d = std::stod(w[idx[q]]);
                    if (!(d > -1e9 && d < 1e9)) return fail("a Radios/rois entry is out of range");
                    cur[q] = static_cast<int>(d);
                }
            } catch (const std::exception &) {
                return fail("a Radios/rois entry is unreadable");
            }
            if (k == 0) {
                bl[0] = cur[0]; bl[1] = cur[1]; tr[0] = cur[2]; tr[1] = cur[3];
            } else if (bl[0] != cur[0] || bl[1] != cur[1] || tr[0] != cur[2] || tr[1] != cur[3]) {
                return fail("the ROI differs between views");
            }
        }
        auto clampi = [](int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); };
        bl[0] = clampi(bl[0], 0, det_px.x - 1);
        bl[1] = clampi(bl[1], 0, det_px.y - 1);
        tr[0] = clampi(tr[0], 0, det_px.x - 1);
        tr[1] = clampi(tr[1], 0, det_px.y - 1);
        m_roiSize = {tr[0] - bl[0] + 1, tr[1] - bl[1] + 1};
        m_roiBLPixel = {bl[0], bl[1]};
        for (const auto &d : det_bl) {
            float x = d.x, y = d.y;
            for (int k = 0; k < bl[0]; ++k) x += m_pixel.x;
            for (int k = 0; k < bl[1]; ++k) y += m_pixel.y;
            m_roiBL.push_back({x, y});
        }
        // every position, spacing and pitch must be a finite float; spacings
        // and pitches positive
        auto fin = [](float a) { return std::isfinite(a); };
        if (!fin(m_fulcrum.x) || !fin(m_fulcrum.y) || !fin(m_fulcrum.z) || !fin(m_detZ))
            return fail("non-finite fulcrum or detector position");
        if (!(fin(m_spacing.x) && fin(m_spacing.y) && fin(m_spacing.z) && m_spacing.x > 0.f && m_spacing.y > 0.f &&
              m_spacing.z > 0.f))
            return fail("Grid/scale must be positive finite spacings");
        if (!(fin(m_pixel.x) && fin(m_pixel.y) && m_pixel.x > 0.f && m_pixel.y > 0.f))
            return fail("Camera extent / pixel count must give a positive finite pitch");
        for (const auto &s : sources)
            if (!fin(s.x) || !fin(s.y) || !fin(s.z)) return fail("non-finite source position");
        for (const auto &r : m_roiBL)
            if (!fin(r.x) || !fin(r.y)) return fail("non-finite detector reference");
        set_sources(sources);
        m_roiPixel = m_pixel;
        m_detBL = det_bl;
        m_detSize = det_px;
        m_blf = centred_corner();
        return true;
    }

    // largest voxel or pixel count per axis read from a file
    static constexpr int kMaxAxis = 1 << 20;

public:

    // volume: voxel counts and spacing, centred at the origin
    // sources: per-view positions (their x and z are averaged, as TomoTable
    //          does, TomoTable.cpp:4-19)
    // roiBottomLeft: per-view ROI bottom-left corner (x, y); detectorZ: one plane
    // roiSize / pixelSpacing: ROI pixel counts and pitch; fulcrum: rotation centre
    TomoGeometry(Size3D volumeSize, VoxelSpacing spacing, const std::vector<Position3D> &sources,
                 const std::vector<Position2D> &roiBottomLeft, float detectorZ, Size2D roiSize,
                 PixelSpacing pixelSpacing, WSize3D fulcrum = {})
        : m_size(volumeSize), m_spacing(spacing), m_roiBL(roiBottomLeft), m_roiSize(roiSize),
          m_pixel(pixelSpacing), m_roiPixel(pixelSpacing), m_fulcrum(fulcrum), m_detZ(detectorZ) {
        if (sources.size() != roiBottomLeft.size() || sources.empty())
            throw std::invalid_argument("TomoGeometry: one source and one ROI origin per view");
        set_sources(sources);
        // built from values, the detector is taken to be the ROI
        m_detWSize = {pixelSpacing.x * static_cast<float>(roiSize.x), pixelSpacing.y * static_cast<float>(roiSize.y)};
        m_detBL = roiBottomLeft;
        m_detSize = roiSize;
        m_blf = centred_corner();
        m_valid = true;
    }

    // TomoGeometry::PerformCheatingAdaptationsForDemonstration
    // (TomoGeometry.cpp:593-611), which the reference's reconstruction main
    // applies after reading a geometry file.  It drops the listed views
    // (indices taken in decreasing order, out-of-range ones skipped; the
    // common source x and z stay the means over all the views read), gives
    // the volume 100 slices of the same spacing, and resamples the detector
    // and its ROI to 3048 x 3048 pixels: the detector pitch, the one the
    // projector uses, becomes the detector's width / 3048, while the ROI
    // corners and the ROI's own pitch keep their values.  As in the
    // reference the volume keeps its bottom-left-front corner, so that after
    // the change of slice count it is no longer centred in z (its positions
    // say so; the projector, in both, treats every volume as centred).
    void PerformCheatingAdaptationsForDemonstration(const std::vector<int> &p_dataIndicesToRemove) {
        auto indices = p_dataIndicesToRemove;
        std::sort(indices.begin(), indices.end(), std::greater<int>());
        for (int i : indices)
            if (i >= 0 && i < static_cast<int>(m_srcY.size())) m_srcY.erase(m_srcY.begin() + i);
        for (int i : indices)
            if (i >= 0 && i < static_cast<int>(m_roiBL.size())) m_roiBL.erase(m_roiBL.begin() + i);
        for (int i : indices)
            if (i >= 0 && i < static_cast<int>(m_detBL.size())) m_detBL.erase(m_detBL.begin() + i);
        m_size.z = 100;
        if (m_detSize.x != 3048 || m_detSize.y != 3048) {
            m_detSize = {3048, 3048};
            m_pixel = {m_detWSize.x / 3048.f, m_detWSize.y / 3048.f};
        }
        m_roiSize = {3048, 3048};
    }
    bool IsValid() const { return m_valid; }
    const std::string &ErrorMessage() const { return m_error; }

    std::vector<float> sourcesYPositions() const { return m_srcY; }
    float sourcesXCommonPosition() const { return m_srcX; }
    float sourcesZCommonPosition() const { return m_srcZ; }
    float detectorsZCommonPosition() const { return m_detZ; }
    float sid() const { return std::abs(m_detZ - m_srcZ); }
    int nbProjections() const { return static_cast<int>(m_srcY.size()); }
    int nbProjectionsRois() const { return nbProjections(); }
    std::vector<Position2D> projectionsRoisBottomLeftPositions() const { return m_roiBL; }
    Size2D projectionsRoisSize() const { return m_roiSize; }
    // The ROI's bottom-left pixel on the full detector (TomoGeometry.h, used
    // by DICOMReader to crop the raw images); {0, 0} unless read from a
    // geometry file or set.
    Size2D GetProjectionROIsBLPixelPositionOnDetector() const { return m_roiBLPixel; }
    void SetProjectionROIsBLPixelPositionOnDetector(Size2D p) { m_roiBLPixel = p; }
    PixelSpacing projectionsPixelSpacing() const { return m_pixel; }
    PixelSpacing projectionsRoisPixelSpacing() const { return m_roiPixel; }
    Size3D volumeSize3D() const { return m_size; }
    VoxelSpacing volumeVoxelSpacing() const { return m_spacing; }
    // The volume (TomoVolume): extent = count x spacing in float, the
    // bottom-left-front corner at minus half the extent when read or built
    // (a centred volume); voxel-corner positions along each axis by repeated
    // float addition of the spacing from that corner; the grid z-major (x
    // fastest).
    WSize3D volumeWSize3D() const {
        return {static_cast<float>(m_size.x) * m_spacing.x, static_cast<float>(m_size.y) * m_spacing.y,
                static_cast<float>(m_size.z) * m_spacing.z};
    }
    Position3D volumeBLF() const { return m_blf; }
    Position3D volumeTRB() const {
        const WSize3D w = volumeWSize3D();
        const Position3D b = volumeBLF();
        return {b.x + w.x, b.y + w.y, b.z + w.z};
    }
    float volumeSize() const {
        const WSize3D w = volumeWSize3D();
        return w.x * w.y * w.z;
    }
    std::vector<float> volumeXs() const { return kvtomo_detail::axis_positions(volumeBLF().x, m_spacing.x, m_size.x); }
    std::vector<float> volumeYs() const { return kvtomo_detail::axis_positions(volumeBLF().y, m_spacing.y, m_size.y); }
    std::vector<float> volumeZs() const { return kvtomo_detail::axis_positions(volumeBLF().z, m_spacing.z, m_size.z); }
    std::vector<Position3D> volumeGridPositions() const {
        const auto xs = volumeXs(), ys = volumeYs(), zs = volumeZs();
        std::vector<Position3D> out;
        out.reserve(xs.size() * ys.size() * zs.size());
        for (float z : zs)
            for (float y : ys)
                for (float x : xs) out.push_back({x, y, z});
        return out;
    }
    std::vector<int> volumeVoxelsIndices() const {
        return kvtomo_detail::indices(static_cast<size_t>(m_size.x) * m_size.y * m_size.z);
    }

    // The full detector and its ROI (TomoProjectionsSet): per view a
    // bottom-left corner, a pixel count and pitch, the extent; pixel
    // positions by repeated float addition of the pitch from the corner.
    std::vector<Position2D> projectionsBottomLeftPositions() const { return m_detBL; }
    Size2D projectionsSize() const { return m_detSize; }
    WSize2D projectionsWSize() const { return m_detWSize; }
    std::vector<std::vector<float>> projectionsXPositions() const {
        return kvtomo_detail::view_positions(m_detBL, true, m_pixel.x, m_detSize.x);
    }
    std::vector<std::vector<float>> projectionsYPositions() const {
        return kvtomo_detail::view_positions(m_detBL, false, m_pixel.y, m_detSize.y);
    }
    std::vector<Position2D> projectionsPositions() const {
        return kvtomo_detail::pixel_positions(projectionsXPositions(), projectionsYPositions());
    }
    std::vector<int> projectionsPositionsIndices() const {
        return kvtomo_detail::indices(m_detBL.size() * static_cast<size_t>(m_detSize.x) * m_detSize.y);
    }
    WSize2D projectionsRoisWSize() const {
        return {static_cast<float>(m_roiSize.x) * m_roiPixel.x, static_cast<float>(m_roiSize.y) * m_roiPixel.y};
    }
    std::vector<std::vector<float>> projectionsRoisXPositions() const {
        return kvtomo_detail::view_positions(m_roiBL, true, m_roiPixel.x, m_roiSize.x);
    }
    std::vector<std::vector<float>> projectionsRoisYPositions() const {
        return kvtomo_detail::view_positions(m_roiBL, false, m_roiPixel.y, m_roiSize.y);
    }
    std::vector<Position2D> projectionsRoisPositions() const {
        return kvtomo_detail::pixel_positions(projectionsRoisXPositions(), projectionsRoisYPositions());
    }
    std::vector<int> projectionsRoisPositionsIndices() const {
        return kvtomo_detail::indices(m_roiBL.size() * static_cast<size_t>(m_roiSize.x) * m_roiSize.y);
    }
    WSize3D fulcrum() const { return m_fulcrum; }
    WSize3D rotationCenter() const { return m_fulcrum; }
    // the geometry file read ("" when built from values)
    std::string filePath() const { return m_filePath; }

    // The parts (TomoGeometry.h:86-89), as read-only views owned by this
    // geometry: valid while it lives, and they read its current values.
    TomoVolume *GetVolume() const {
        m_volumeView = TomoVolume(this);
        return &m_volumeView;
    }
    TomoProjectionsSet *GetProjections() const {
        m_projectionsView = TomoProjectionsSet(this, false);
        return &m_projectionsView;
    }
    TomoProjectionsSet *GetProjectionsRois() const {
        m_roisView = TomoProjectionsSet(this, true);
        return &m_roisView;
    }
    TomoTable *GetTable() const {
        m_tableView = TomoTable(this);
        return &m_tableView;
    }

    // Flattened description the kernels consume (Projector.cu:917-940):
    // sources (common x, y_i, common z), ROI origins (x_i, y_i, common z).
    struct Flat {
        kv_geometry g;
        std::vector<float> src, det;
    };
    std::shared_ptr<Flat> flatten() const {
        auto f = std::make_shared<Flat>();
        const int P = nbProjections();
        f->src.resize(3 * P);
        f->det.resize(3 * P);
        for (int i = 0; i < P; ++i) {
            f->src[3 * i] = m_srcX;
            f->src[3 * i + 1] = m_srcY[i];
            f->src[3 * i + 2] = m_srcZ;
            f->det[3 * i] = m_roiBL[i].x;
            f->det[3 * i + 1] = m_roiBL[i].y;
            f->det[3 * i + 2] = m_detZ;
        }
        f->g = kv_geometry{m_size.x, m_size.y, m_size.z, m_spacing.x, m_spacing.y, m_spacing.z, P,
                           m_roiSize.x, m_roiSize.y, m_pixel.x, m_pixel.y, f->src.data(), f->det.data(),
                           m_fulcrum.z};
        return f;
    }

private:
    Position3D centred_corner() const {
        const WSize3D w = volumeWSize3D();
        return {-0.5f * w.x, -0.5f * w.y, -0.5f * w.z};
    }

    // common source x and z: float sums over the views (TomoTable.cpp:4-19)
    void set_sources(const std::vector<Position3D> &sources) {
        float sx = 0.f, sz = 0.f;
        m_srcY.clear();
        for (const auto &s : sources) {
            sx += s.x;
            m_srcY.push_back(s.y);
            sz += s.z;
        }
        m_srcX = sx / static_cast<float>(sources.size());
        m_srcZ = sz / static_cast<float>(sources.size());
    }

    Size3D m_size;
    VoxelSpacing m_spacing;
    std::vector<float> m_srcY;
    float m_srcX = 0.f, m_srcZ = 0.f;
    std::vector<Position2D> m_roiBL;
    Size2D m_roiSize;
    Size2D m_roiBLPixel;
    PixelSpacing m_pixel;     // detector pitch (what the projector uses)
    PixelSpacing m_roiPixel;  // the ROI set's own pitch
    WSize2D m_detWSize;       // detector extent (mm)
    std::vector<Position2D> m_detBL;  // per-view detector bottom-left corners
    Position3D m_blf;         // the volume's bottom-left-front corner
    Size2D m_detSize;         // detector pixel counts
    WSize3D m_fulcrum;
    float m_detZ = 0.f;
    bool m_valid = false;
    std::string m_error;
    std::string m_filePath;
    mutable TomoVolume m_volumeView;
    mutable TomoProjectionsSet m_projectionsView, m_roisView;
    mutable TomoTable m_tableView;
};

inline int TomoVolume::GetVoxelsNumber() const {
    const Size3D n = m_g->volumeSize3D();
    return n.x * n.y * n.z;
}
inline float TomoVolume::GetSize() const { return m_g->volumeSize(); }
inline Size3D TomoVolume::GetSize3D() const { return m_g->volumeSize3D(); }
inline WSize3D TomoVolume::GetWSize3D() const { return m_g->volumeWSize3D(); }
inline Position3D TomoVolume::GetBottomLeftFront() const { return m_g->volumeBLF(); }
inline Position3D TomoVolume::GetTopRightBack() const { return m_g->volumeTRB(); }
inline VoxelSpacing TomoVolume::GetVoxelSpacing() const { return m_g->volumeVoxelSpacing(); }
inline std::vector<float> TomoVolume::GetXPositions() const { return m_g->volumeXs(); }
inline std::vector<float> TomoVolume::GetYPositions() const { return m_g->volumeYs(); }
inline std::vector<float> TomoVolume::GetZPositions() const { return m_g->volumeZs(); }
inline std::vector<Position3D> TomoVolume::GetGridPositions() const { return m_g->volumeGridPositions(); }
inline std::vector<int> TomoVolume::GetVoxelsIndices() const { return m_g->volumeVoxelsIndices(); }

inline std::vector<Position2D> TomoProjectionsSet::GetBottomLeftPositions() const {
    return m_rois ? m_g->projectionsRoisBottomLeftPositions() : m_g->projectionsBottomLeftPositions();
}
inline Size2D TomoProjectionsSet::GetSize() const {
    return m_rois ? m_g->projectionsRoisSize() : m_g->projectionsSize();
}
inline WSize2D TomoProjectionsSet::GetWSize() const {
    return m_rois ? m_g->projectionsRoisWSize() : m_g->projectionsWSize();
}
inline PixelSpacing TomoProjectionsSet::GetPixelSpacing() const {
    return m_rois ? m_g->projectionsRoisPixelSpacing() : m_g->projectionsPixelSpacing();
}
inline std::vector<std::vector<float>> TomoProjectionsSet::GetXPositions() const {
    return m_rois ? m_g->projectionsRoisXPositions() : m_g->projectionsXPositions();
}
inline std::vector<std::vector<float>> TomoProjectionsSet::GetYPositions() const {
    return m_rois ? m_g->projectionsRoisYPositions() : m_g->projectionsYPositions();
}
inline std::vector<Position2D> TomoProjectionsSet::GetProjectionPositions() const {
    return m_rois ? m_g->projectionsRoisPositions() : m_g->projectionsPositions();
}
inline std::vector<int> TomoProjectionsSet::GetProjectionPixelsIndices() const {
    return m_rois ? m_g->projectionsRoisPositionsIndices() : m_g->projectionsPositionsIndices();
}
inline int TomoProjectionsSet::GetNProjections() const {
    return static_cast<int>(GetBottomLeftPositions().size());
}

inline int TomoTable::GetSourcesNumber() const { return m_g->nbProjections(); }
inline std::vector<float> TomoTable::GetSourcesYPositions() const { return m_g->sourcesYPositions(); }
inline float TomoTable::GetSourcesXCommonPosition() const { return m_g->sourcesXCommonPosition(); }
inline float TomoTable::GetSourcesZCommonPosition() const { return m_g->sourcesZCommonPosition(); }
inline float TomoTable::GetDetectorsZCommonPosition() const { return m_g->detectorsZCommonPosition(); }

// A readable summary under the reference printer's headings
// (TomoGeometry.h:119-125): volume, projections, projections Rois, table.
inline std::ostream &operator<<(std::ostream &os, TomoGeometry const &g) {
    const auto n = g.volumeSize3D();
    const auto d = g.volumeVoxelSpacing();
    const auto roi = g.projectionsRoisSize();
    const auto px = g.projectionsPixelSpacing();
    os << "volume " << n.x << " x " << n.y << " x " << n.z << " voxels of " << d.x << " x " << d.y << " x " << d.z
       << " mm, centred at the origin" << std::endl;
    os << "projections: " << g.nbProjections() << " views, pixel pitch " << px.x << " x " << px.y << " mm" << std::endl;
    os << "projections Rois: " << roi.x << " x " << roi.y << " pixels, bottom-left corners";
    for (const auto &b : g.projectionsRoisBottomLeftPositions()) os << " (" << b.x << ", " << b.y << ")";
    os << std::endl;
    os << "table: sources x " << g.sourcesXCommonPosition() << ", z " << g.sourcesZCommonPosition() << ", y";
    for (float y : g.sourcesYPositions()) os << " " << y;
    os << "; detector z " << g.detectorsZCommonPosition() << std::endl;
    return os;
}

// ---------------------------------------------------------------- engine

namespace kvtomo_detail {
// One context per host thread, created on first use.
inline kv_ctx *thread_context() {
    struct Holder {
        kv_ctx *ctx = nullptr;
        ~Holder() {
            if (ctx) kv_ctx_destroy(ctx);
        }
    };
    thread_local Holder h;
    if (h.ctx == nullptr) {
        const char *dev = std::getenv("KVTOMO_DEVICE");
        if (kv_ctx_create(dev ? std::atoi(dev) : 0, &h.ctx) != KV_OK) h.ctx = nullptr;
    }
    return h.ctx;
}

struct PlanHandle {
    kv_plan *plan = nullptr;
    ~PlanHandle() {
        if (plan) kv_plan_destroy(plan);
    }
};

inline std::shared_ptr<PlanHandle> make_plan(const TomoGeometry *g, kv_family family,
                                              kv_storage storage = KV_STORAGE_F32) {
    kv_ctx *ctx = thread_context();
    if (ctx == nullptr || g == nullptr) return nullptr;
    auto flat = g->flatten();
    auto h = std::make_shared<PlanHandle>();
    if (kv_plan_create(ctx, &flat->g, family, storage, &h->plan) != KV_OK) return nullptr;
    return h;
}

}  // namespace kvtomo_detail

namespace kvtomo_detail {

// Baseline TIFF, little endian, uncompressed, one strip per page, one page
// per z slice; samples of `bytes` bytes, SampleFormat 1 (unsigned) or 3 (IEEE).
inline bool write_tiff_pages(const std::string &path, int w, int h, int pages, int bytes, int sample_format,
                             const uint8_t *data) {
    const int ntags = 11;
    const uint32_t ifd_bytes = 2 + ntags * 12 + 4;
    // classic TIFF: 32-bit offsets, so the whole file must stay below 4 GiB
    if (w <= 0 || h <= 0 || pages <= 0 || data == nullptr) return false;
    const uint64_t total = 8 + (uint64_t)pages * (ifd_bytes + (uint64_t)w * h * bytes);
    if (total >= (1ull << 32)) return false;
    const uint32_t page_bytes = (uint32_t)w * h * bytes;
    std::ofstream f(path, std::ios::binary);
    if (!f) return false;
    auto put16 = [&](uint16_t v) { f.put((char)(v & 0xFF)); f.put((char)(v >> 8)); };
    auto put32 = [&](uint32_t v) { for (int i = 0; i < 4; ++i) f.put((char)((v >> (8 * i)) & 0xFF)); };
    f.write("II", 2);
    put16(42);
    put32(8);                                    // first IFD right after the header
    uint32_t off = 8;
    for (int p = 0; p < pages; ++p) {
        const uint32_t data_off = off + ifd_bytes;
        const uint32_t next = p + 1 < pages ? data_off + page_bytes : 0;
        put16(ntags);
        auto tag = [&](uint16_t t, uint16_t type, uint32_t count, uint32_t value) {
            put16(t); put16(type); put32(count);
            if (type == 3 && count == 1) { put16((uint16_t)value); put16(0); }
            else put32(value);
        };
        tag(256, 4, 1, (uint32_t)w);             // ImageWidth
        tag(257, 4, 1, (uint32_t)h);             // ImageLength
        tag(258, 3, 1, (uint32_t)(8 * bytes));   // BitsPerSample
        tag(259, 3, 1, 1);                       // Compression: none
        tag(262, 3, 1, 1);                       // Photometric: black is zero
        tag(273, 4, 1, data_off);                // StripOffsets
        tag(277, 3, 1, 1);                       // SamplesPerPixel
        tag(278, 4, 1, (uint32_t)h);             // RowsPerStrip
        tag(279, 4, 1, page_bytes);              // StripByteCounts
        tag(284, 3, 1, 1);                       // PlanarConfiguration: contiguous
        tag(339, 3, 1, (uint32_t)sample_format); // SampleFormat
        put32(next);
        // rows top first: memory row h-1 is the image's top row
        const uint8_t *page = data + (size_t)p * page_bytes;
        for (int y = h - 1; y >= 0; --y) f.write(reinterpret_cast<const char *>(page + (size_t)y * w * bytes), (std::streamsize)w * bytes);
        off = data_off + page_bytes;
    }
    return (bool)f;
}

}  // namespace kvtomo_detail

// Float32 volume (or projection stack) to a multi-page TIFF.
inline bool WriteTIFF(const std::string &path, const ImageDataPtr &img) {
    const int *d = img->GetDimensions();
    return kvtomo_detail::write_tiff_pages(path, d[0], d[1], d[2], 4, 3,
                                           reinterpret_cast<const uint8_t *>(img->data()));
}


class Projector {
public:
    Projector(TomoGeometry *p_tomoGeometry, kv_family family = KV_FAMILY_RC)
        : m_tomoGeometry(p_tomoGeometry), m_family(family) {}

    // Projector::PerformProjection, Projector.cu:873-1036.  Returns nullptr on failure.
    ImageDataPtr PerformProjection(ImageDataPtr p_volume) const {
        if (!ensure() || p_volume == nullptr || p_volume->size() != kv_plan_volume_elems(m_plan->plan)) return nullptr;
        auto out = ImageData::New();
        const auto roi = m_tomoGeometry->projectionsRoisSize();
        out->SetDimensions(roi.x, roi.y, m_tomoGeometry->nbProjectionsRois());
        out->SetSpacing(m_tomoGeometry->projectionsPixelSpacing().x, m_tomoGeometry->projectionsPixelSpacing().y, 1.);
        out->AllocateScalars();
        if (kv_forward(m_plan->plan, p_volume->data(), out->data(), KV_MEM_HOST) != KV_OK) return nullptr;
        return out;
    }

    // Single-view projection into an existing container (Projector.cu:823-870,
    // unfinished in the reference): the container's ROI origin is the
    // geometry's first ROI corner on the common detector plane.
    void PerformProjection(const ImageDataPtr p_volume, const Position3D &p_sourcePosition,
                           ImageDataPtr p_projectionsContainer) const {
        if (!ensure() || p_volume == nullptr || p_projectionsContainer == nullptr) return;
        const auto roi = m_tomoGeometry->projectionsRoisSize();
        if (p_projectionsContainer->size() != (size_t)roi.x * roi.y) {
            p_projectionsContainer->SetDimensions(roi.x, roi.y, 1);
            p_projectionsContainer->AllocateScalars();
        }
        const auto bl = m_tomoGeometry->projectionsRoisBottomLeftPositions().front();
        const float src[3] = {p_sourcePosition.x, p_sourcePosition.y, p_sourcePosition.z};
        const float det[3] = {bl.x, bl.y, m_tomoGeometry->detectorsZCommonPosition()};
        kv_forward_single(m_plan->plan, p_volume->data(), src, det, p_projectionsContainer->data(), KV_MEM_HOST);
    }

    // Projector::PerformBackProjection, Projector.cu:1038-1207.
    ImageDataPtr PerformBackProjection(ImageDataPtr p_projections) const {
        if (!ensure() || p_projections == nullptr || p_projections->size() != kv_plan_proj_elems(m_plan->plan))
            return nullptr;
        auto out = ImageData::New();
        const auto n = m_tomoGeometry->volumeSize3D();
        const auto s = m_tomoGeometry->volumeVoxelSpacing();
        out->SetDimensions(n.x, n.y, n.z);
        out->SetSpacing(s.x, s.y, s.z);
        out->AllocateScalars();
        if (kv_back(m_plan->plan, p_projections->data(), out->data(), KV_MEM_HOST) != KV_OK) return nullptr;
        return out;
    }

    kv_plan *plan() const { return ensure() ? m_plan->plan : nullptr; }

private:
    bool ensure() const {
        if (!m_plan) m_plan = kvtomo_detail::make_plan(m_tomoGeometry, m_family);
        return m_plan != nullptr;
    }
    TomoGeometry *m_tomoGeometry;
    kv_family m_family;
    mutable std::shared_ptr<kvtomo_detail::PlanHandle> m_plan;
};

namespace recons {

namespace detail {
inline ImageDataPtr uniform_volume(const TomoGeometry *g) {
    // PhantomMaker(volume, 1.f).GetPhantom(): background density 1 everywhere
    auto v = ImageData::New();
    const auto n = g->volumeSize3D();
    const auto s = g->volumeVoxelSpacing();
    v->SetDimensions(n.x, n.y, n.z);
    v->SetSpacing(s.x, s.y, s.z);
    v->AllocateScalars();
    for (size_t i = 0; i < v->size(); ++i) v->data()[i] = 1.f;
    return v;
}

inline Result<ImageDataPtr> iterate(bool mlem, TomoGeometry *g, ImageDataPtr proj, int iters, float relax,
                                    std::optional<ImageDataPtr> init, std::optional<std::string> outDir,
                                    kv_family family) {
    // the reference reports MLEM failures with the ART code (Reconstructors.h:159,190,230)
    const auto code = ReconstructorsErrorCode::ART;
    ImageDataPtr x = init.has_value() ? init.value() : uniform_volume(g);
    if (x == nullptr || proj == nullptr) return code;
    Projector projector(g, family);
    kv_plan *plan = projector.plan();
    if (plan == nullptr || x->size() != kv_plan_volume_elems(plan) || proj->size() != kv_plan_proj_elems(plan))
        return code;
    auto run = mlem ? kv_mlem : kv_sart;
    if (!outDir.has_value()) {
        if (run(plan, proj->data(), x->data(), iters, relax, KV_MEM_HOST, nullptr, nullptr) != KV_OK) return code;
        return x;
    }
    // verbose mode, with the reference's files (Reconstructors.h:47-131,
    // 164-248) as multi-page TIFFs: the initial volume; per iteration the
    // projection A x, the corrected projection -- relax (p - A x) for ART,
    // relax p / A x where A x is not zero (AlmostEqualRelative, float
    // epsilon) and A x elsewhere for MLEM -- and the new iterate.  The fused
    // kernels keep the projections on the device, so in this mode each
    // iteration runs one extra forward projection to the host for the dumps.
    const std::string dir = outDir.value();
    WriteTIFF(dir + "initialVolume.tiff", x);
    for (int it = 0; it < iters; ++it) {
        const std::string step = std::to_string(it) + ".tiff";
        ImageDataPtr q = projector.PerformProjection(x);
        if (q == nullptr) return code;
        WriteTIFF(dir + "currentProjectionStep" + step, q);
        const float *p = proj->data();
        float *c = q->data();
        const float eps = std::numeric_limits<float>::epsilon();
        for (size_t i = 0; i < q->size(); ++i) {
            if (!mlem) c[i] = relax * (p[i] - c[i]);
            else if (!(std::fabs(c[i]) <= eps * std::fabs(c[i]))) c[i] = relax * (p[i] / c[i]);
        }
        WriteTIFF(dir + "currentCorrectedProjectionStep" + step, q);
        if (run(plan, proj->data(), x->data(), 1, relax, KV_MEM_HOST, nullptr, nullptr) != KV_OK) return code;
        WriteTIFF(dir + "reconstructionstep" + step, x);
    }
    return x;
}
}  // namespace detail

// recons::ART, Reconstructors.h:19-134 (simultaneous: x += B(relax (p - A x)))
inline Result<ImageDataPtr> ART(TomoGeometry *p_tomoGeometry, ImageDataPtr p_projectionImages,
                                int p_iterationNumber, float p_relaxationCoefficient,
                                std::optional<ImageDataPtr> p_initialVolume,
                                std::optional<std::string> p_outputDirectoryPath,
                                kv_family family = KV_FAMILY_RC) {
    return detail::iterate(false, p_tomoGeometry, p_projectionImages, p_iterationNumber, p_relaxationCoefficient,
                           p_initialVolume, p_outputDirectoryPath, family);
}

// recons::MLEM, Reconstructors.h:136-253 (x *= B(relax p / A x))
inline Result<ImageDataPtr> MLEM(TomoGeometry *p_tomoGeometry, ImageDataPtr p_projectionImages,
                                 int p_iterationNumber, float p_relaxationCoefficient,
                                 std::optional<ImageDataPtr> p_initialVolume,
                                 std::optional<std::string> p_outputDirectoryPath,
                                 kv_family family = KV_FAMILY_RC) {
    return detail::iterate(true, p_tomoGeometry, p_projectionImages, p_iterationNumber, p_relaxationCoefficient,
                           p_initialVolume, p_outputDirectoryPath, family);
}

// recons::BackProjection, Reconstructors.h:256-261
inline Result<ImageDataPtr> BackProjection(TomoGeometry *p_tomoGeometry, ImageDataPtr p_projectionImages,
                                           kv_family family = KV_FAMILY_RC) {
    Projector projector{p_tomoGeometry, family};
    auto out = projector.PerformBackProjection(p_projectionImages);
    if (out == nullptr) return ReconstructorsErrorCode::BackProjectionFailed;
    return out;
}

// Filtered backprojection (kv_fbp): Shepp-Logan ramp along the sweep
// direction, exact transpose, sensitivity normalisation.  No reference
// counterpart (the reference's "FBP" reconstructor backprojects unfiltered
// data); always the EXACT family.
inline Result<ImageDataPtr> FilteredBackProjection(TomoGeometry *p_tomoGeometry, ImageDataPtr p_projectionImages,
                                                   int p_halfTaps = 128) {
    if (p_tomoGeometry == nullptr || p_projectionImages == nullptr)
        return ReconstructorsErrorCode::BackProjectionFailed;
    Projector projector{p_tomoGeometry, KV_FAMILY_EXACT};
    kv_plan *plan = projector.plan();
    if (plan == nullptr || p_projectionImages->size() != kv_plan_proj_elems(plan))
        return ReconstructorsErrorCode::BackProjectionFailed;
    auto out = ImageData::New();
    const auto sz = p_tomoGeometry->volumeSize3D();
    const auto sp = p_tomoGeometry->volumeVoxelSpacing();
    out->SetDimensions(sz.x, sz.y, sz.z);
    out->SetSpacing(sp.x, sp.y, sp.z);
    out->AllocateScalars();
    if (kv_fbp(plan, p_projectionImages->data(), out->data(), p_halfTaps, KV_MEM_HOST) != KV_OK)
        return ReconstructorsErrorCode::BackProjectionFailed;
    return out;
}

// recons::ShiftAndAdd, Reconstructors.h:263-379: one detector-sized slice per
// volume slice.  Verbose mode (an output directory given) prints the fulcrum
// height and the source-to-image distance, as the reference does; it writes
// no files.
inline Result<ImageDataPtr> ShiftAndAdd(TomoGeometry *p_tomoGeometry, ImageDataPtr p_projectionImages,
                                        std::optional<std::string> p_outputDirectoryPath = std::nullopt,
                                        kv_family family = KV_FAMILY_RC) {
    if (p_tomoGeometry == nullptr || p_projectionImages == nullptr) return ReconstructorsErrorCode::ShiftAndAdd;
    if (p_outputDirectoryPath.has_value()) {
        std::cout << "zF = " << std::to_string(p_tomoGeometry->fulcrum().z) << std::endl;
        std::cout << "sid = " << std::to_string(p_tomoGeometry->sid()) << std::endl;
    }
    Projector projector{p_tomoGeometry, family};
    kv_plan *plan = projector.plan();
    if (plan == nullptr || p_projectionImages->size() != kv_plan_proj_elems(plan))
        return ReconstructorsErrorCode::ShiftAndAdd;
    auto out = ImageData::New();
    const auto roi = p_tomoGeometry->projectionsRoisSize();
    out->SetDimensions(roi.x, roi.y, p_tomoGeometry->volumeSize3D().z);
    out->AllocateScalars();
    if (kv_shift_and_add(plan, p_projectionImages->data(), out->data(), KV_MEM_HOST) != KV_OK)
        return ReconstructorsErrorCode::ShiftAndAdd;
    return out;
}

}  // namespace recons
