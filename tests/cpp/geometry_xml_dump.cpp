// Reads a geometry file with the drop-in header's TomoGeometry(path) and
// prints the flattened description the kernels receive, as JSON.  With
// "adapt i j ..." after the path it first applies
// PerformCheatingAdaptationsForDemonstration({i, j, ...}).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "kevernals_tomo.hpp"

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
    if (argc < 2) return 2;
    TomoGeometry geo{std::string(argv[1])};
    if (!geo.IsValid()) {
        std::printf("{\"valid\": false, \"error\": \"%s\"}\n", json_escape(geo.ErrorMessage()).c_str());
        return 0;
    }
    if (argc > 2 && std::string(argv[2]) == "adapt") {
        std::vector<int> remove;
        for (int i = 3; i < argc; ++i) remove.push_back(std::atoi(argv[i]));
        geo.PerformCheatingAdaptationsForDemonstration(remove);
    }
    const auto f = geo.flatten();
    const kv_geometry &g = f->g;
    std::printf("{\"valid\": true, \"n\": [%d, %d, %d], \"d\": [%.9g, %.9g, %.9g], \"views\": %d, "
                "\"det\": [%d, %d], \"pitch\": [%.9g, %.9g], \"fulcrum_z\": %.9g, \"src\": [",
                g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.n_views, g.nu, g.nv, g.du, g.dv, g.fulcrum_z);
    for (int i = 0; i < 3 * g.n_views; ++i) std::printf("%s%.9g", i ? ", " : "", g.src[i]);
    std::printf("], \"det_origin\": [");
    for (int i = 0; i < 3 * g.n_views; ++i) std::printf("%s%.9g", i ? ", " : "", g.det_origin[i]);
    std::printf("]}\n");
    return 0;
}
