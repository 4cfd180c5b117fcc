// emst_io.cu -- the reference's point and result files (host code only).
//
// Readers follow InputRW.h:60-623 (emst_coalition/include): the suffix picks the
// format -- ".2d" (count, then "x y" per point), ".3d" (count, then "x y z"),
// ".points" ("Width = W Height = H", then "x y z" per point), anything else
// TSPLIB ("NODE_COORD_SECTION", then "i x y" per point; DIMENSION gives the
// count).  Coordinates are read as float, as the reference does.
//
// Writers follow NeuralNetEMST.h:275-326 and BufferLink.h:266-279 (writeLinks)
// and the grid writers (GridOfNodes.h): "<base>.links" holds, per point, its
// tree neighbours as "j 0" pairs; "<base>.disjointSetMap" the final root of
// each point as the byte offset of a 4-byte label (4 x root id);
// "<base>.points" the rescaled coordinates (x y z, z = 0 in 2D) at the default
// 6 significant digits.  Neighbours are written by Boruvka round, then by id:
// the reference inserts links from concurrent threads, so its order within a
// record is not reproducible anyway; files compare as neighbour sets.
#include <algorithm>
#include <cctype>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/emst.h"

namespace {

std::string suffix_of(const std::string& path)
{
    // the file name's extension (directories may hold dots)
    const size_t slash = path.find_last_of("/\\");
    const std::string name = slash == std::string::npos ? path : path.substr(slash + 1);
    const size_t dot = name.find_last_of('.');
    if (dot == std::string::npos) return "";
    std::string s = name.substr(dot);
    for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
    return s;
}

bool read_tsp(std::ifstream& fi, std::vector<float>& out, int64_t& n)
{
    std::string line;
    int64_t dimension = -1;
    while (std::getline(fi, line)) {
        if (line.find("NODE_COORD_SECTION") != std::string::npos) break;
        const size_t p = line.find("DIMENSION");
        if (p != std::string::npos) {
            const size_t c = line.find(':', p);
            dimension = std::atoll(line.c_str() + (c == std::string::npos ? p + 9 : c + 1));
        }
    }
    if (dimension < 0 || !fi) return false;
    out.resize((size_t)dimension * 2);
    for (int64_t i = 0; i < dimension; ++i) {
        long long idx;
        float x, y;
        if (!(fi >> idx >> x >> y)) return false;
        out[2 * i] = x;
        out[2 * i + 1] = y;
    }
    n = dimension;
    return true;
}

bool read_counted(std::ifstream& fi, int dim, std::vector<float>& out, int64_t& n)
{
    long long count;
    if (!(fi >> count) || count < 0) return false;
    out.resize((size_t)count * dim);
    for (long long i = 0; i < count * dim; ++i)
        if (!(fi >> out[i])) return false;
    n = count;
    return true;
}

bool read_points_grid(std::ifstream& fi, std::vector<float>& out, int64_t& n)
{
    std::string w1, w2;
    long long width, height;
    if (!(fi >> w1 >> w2 >> width) || !(fi >> w1 >> w2 >> height) || width < 0 || height < 0) return false;
    const long long count = width * height;
    out.resize((size_t)count * 3);
    for (long long i = 0; i < count * 3; ++i)
        if (!(fi >> out[i])) return false;
    n = count;
    return true;
}

}  // namespace

extern "C" {

emst_status emst_read_points(const char* path, float* points, int64_t cap, int64_t* n, int* dim)
{
    if (!path || !n || !dim) return EMST_EINVAL;
    std::ifstream fi(path);
    if (!fi) return EMST_EINVAL;
    const std::string sfx = suffix_of(path);
    std::vector<float> buf;
    int64_t count = 0;
    int d = 2;
    bool ok;
    if (sfx == ".2d") {
        ok = read_counted(fi, 2, buf, count);
    } else if (sfx == ".3d") {
        d = 3;
        ok = read_counted(fi, 3, buf, count);
    } else if (sfx == ".points") {
        d = 3;
        ok = read_points_grid(fi, buf, count);
    } else {
        ok = read_tsp(fi, buf, count);
    }
    if (!ok) return EMST_EINVAL;
    *n = count;
    *dim = d;
    if (points) {
        if (cap < count) return EMST_EOVERFLOW;
        std::memcpy(points, buf.data(), sizeof(float) * (size_t)count * d);
    }
    return EMST_OK;
}

emst_status emst_write_results(emst_ctx* ctx, const char* base)
{
    if (!ctx || !base) return EMST_EINVAL;
    int64_t n = 0, ne = 0;
    int dim = 0;
    emst_status st = emst_get_size(ctx, &n, &dim);
    if (st != EMST_OK) return st;
    st = emst_get_edges(ctx, nullptr, nullptr, 0, &ne);  // count only (too-small buffer is expected)
    if (st != EMST_OK && st != EMST_EOVERFLOW) return st;
    std::vector<int32_t> uv((size_t)2 * (ne > 0 ? ne : 1)), rd((size_t)(ne > 0 ? ne : 1));
    if (ne > 0 && (st = emst_get_edges(ctx, uv.data(), rd.data(), ne, &ne)) != EMST_OK) return st;
    std::vector<int32_t> lab((size_t)(n > 0 ? n : 1));
    if (n > 0 && (st = emst_get_labels(ctx, lab.data(), n)) != EMST_OK) return st;
    std::vector<float> sp((size_t)(n > 0 ? n : 1) * dim);
    double ux = 0.0;
    if (n > 0 && (st = emst_get_rescaled(ctx, sp.data(), &ux, n * dim)) != EMST_OK) return st;

    // adjacency: neighbours of each point in (round, id) order
    std::vector<int64_t> deg((size_t)n + 1, 0);
    for (int64_t e = 0; e < ne; ++e) {
        ++deg[uv[2 * e] + 1];
        ++deg[uv[2 * e + 1] + 1];
    }
    for (int64_t i = 0; i < n; ++i) deg[i + 1] += deg[i];
    std::vector<std::pair<int32_t, int32_t>> adj((size_t)deg[n]);  // (round, neighbour)
    std::vector<int64_t> fill(deg.begin(), deg.end() - 1);
    for (int64_t e = 0; e < ne; ++e) {
        const int32_t u = uv[2 * e], v = uv[2 * e + 1];
        adj[fill[u]++] = {rd[e], v};
        adj[fill[v]++] = {rd[e], u};
    }
    const std::string b(base);
    {
        std::ofstream fo(b + ".links");
        if (!fo) return EMST_EINVAL;
        fo << "Width = " << n << " Height = " << 1 << " " << std::endl;
        for (int64_t i = 0; i < n; ++i) {
            std::sort(adj.begin() + deg[i], adj.begin() + deg[i + 1]);
            fo << std::endl << "NodeP = " << i << " " << 0;
            fo << " NumLinks = " << (deg[i + 1] - deg[i]) << " ";
            for (int64_t k = deg[i]; k < deg[i + 1]; ++k) fo << adj[k].second << " " << 0 << " ";
            fo << std::endl;
        }
        if (!fo) return EMST_EINVAL;
    }
    {
        std::ofstream fo(b + ".disjointSetMap");
        if (!fo) return EMST_EINVAL;
        fo << "Width = " << n << " Height = " << 1 << " " << std::endl;
        for (int64_t i = 0; i < n; ++i) fo << (int64_t)lab[i] * 4 << " ";
        fo << std::endl << std::endl;
        if (!fo) return EMST_EINVAL;
    }
    {
        std::ofstream fo(b + ".points");
        if (!fo) return EMST_EINVAL;
        fo << "Width = " << n << " Height = " << 1 << " " << std::endl;
        for (int64_t i = 0; i < n; ++i) {
            fo << sp[i * dim] << " " << sp[i * dim + 1] << " " << (dim == 3 ? sp[i * dim + 2] : 0.f) << " ";
            fo << " ";
        }
        fo << std::endl << std::endl;
        if (!fo) return EMST_EINVAL;
    }
    return EMST_OK;
}

emst_status emst_read_links(const char* path, int32_t* uv, int64_t cap, int64_t* n_edges, int64_t* n_points)
{
    if (!path || !n_edges) return EMST_EINVAL;
    std::ifstream fi(path);
    if (!fi) return EMST_EINVAL;
    std::string w1, w2;
    long long width, height;
    if (!(fi >> w1 >> w2 >> width) || !(fi >> w1 >> w2 >> height)) return EMST_EINVAL;
    std::vector<int32_t> out;
    std::string tok;
    while (fi >> tok) {
        if (tok != "NodeP") continue;
        long long x, y, k;
        std::string eq, nl;
        if (!(fi >> eq >> x >> y >> nl >> eq >> k)) return EMST_EINVAL;
        for (long long j = 0; j < k; ++j) {
            long long nx, ny;
            if (!(fi >> nx >> ny)) return EMST_EINVAL;
            if (x < nx) {  // each undirected edge once
                out.push_back((int32_t)x);
                out.push_back((int32_t)nx);
            }
        }
    }
    *n_edges = (int64_t)out.size() / 2;
    if (n_points) *n_points = width * height;
    if (uv) {
        if (cap < *n_edges) return EMST_EOVERFLOW;
        std::memcpy(uv, out.data(), sizeof(int32_t) * out.size());
    }
    return EMST_OK;
}

}  // extern "C"
