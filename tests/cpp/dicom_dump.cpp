// Reads a DICOM directory with the drop-in's DICOMReader (detector ROI from a
// geometry file) and prints the stacked images and their log(1 + x) as JSON.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "kevernals_dicom.hpp"

// a string as the body of a JSON string literal
static std::string json_escape(const std::string &v) {
    std::string out;
    for (char c : v) {
        if (c == '"' || c == '\\') out += '\\';
        out += c;
    }
    return out;
}

int main(int argc, char **argv) {
    if (argc < 3) return 2;
    TomoGeometry geo{std::string(argv[1])};
    if (!geo.IsValid()) {
        std::printf("{\"ok\": false, \"error\": \"geometry: %s\"}\n", json_escape(geo.ErrorMessage()).c_str());
        return 0;
    }
    std::vector<int> remove;
    for (int i = 3; i < argc; ++i) remove.push_back(std::atoi(argv[i]));
    DICOMReader reader(&geo);
    auto res = reader.ReadDirectory(argv[2], remove);
    if (!res) {
        std::printf("{\"ok\": false, \"error\": \"%s\", \"code\": \"%s\"}\n",
                    json_escape(reader.LastError()).c_str(), json_escape(res.error().message()).c_str());
        return 0;
    }
    const auto img = res.value();
    const auto lg = LogarithmicScale(img);
    const int *d = img->GetDimensions();
    std::printf("{\"ok\": true, \"dims\": [%d, %d, %d], \"data\": [", d[0], d[1], d[2]);
    for (size_t i = 0; i < img->size(); ++i) std::printf("%s%.9g", i ? ", " : "", img->data()[i]);
    std::printf("], \"log\": [");
    for (size_t i = 0; i < lg->size(); ++i) std::printf("%s%.9g", i ? ", " : "", lg->data()[i]);
    std::printf("]}\n");
    return 0;
}
