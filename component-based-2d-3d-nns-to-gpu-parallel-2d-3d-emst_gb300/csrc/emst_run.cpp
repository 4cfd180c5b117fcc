// emst_run -- command-line driver with the reference's argument order
// (emst_coalition/src/main.cpp:19-93): data file, solution file, stats file,
// config file, with the same defaults when arguments are missing.
//
//   emst_run [data [solution [stats [config]]]] [--static] [--device N]
//
// The data file is read like InputRW::readFile (.2d / .3d / .points / TSPLIB),
// the EMST is solved on the GPU, and the solution's base name (the solution
// path without its extension) receives .links, .disjointSetMap and .points,
// as CalculateurEMST::run writes them.  One line is appended to the stats
// file: points, dimension, edges, tree length, rounds, milliseconds.  The
// config file is accepted for argument compatibility; the solver needs no
// parameters from it.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/emst.h"

static std::string base_of(const std::string& path)
{
    const size_t slash = path.find_last_of("/\\");
    const size_t dot = path.find_last_of('.');
    if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return path;
    return path.substr(0, dot);
}

static int fail(emst_ctx* ctx, emst_status st, const char* what)
{
    std::fprintf(stderr, "emst_run: %s failed (status %d)%s%s\n", what, (int)st, ctx ? ": " : "",
                 ctx ? emst_last_error(ctx) : "");
    if (ctx) emst_destroy(ctx);
    return 1;
}

int main(int argc, char** argv)
{
    std::vector<std::string> pos;
    int device = 0;
    bool static_table = false;
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--static")) {
            static_table = true;
        } else if (!std::strcmp(argv[i], "--device") && i + 1 < argc) {
            device = std::atoi(argv[++i]);
        } else {
            pos.push_back(argv[i]);
        }
    }
    const std::string data = pos.size() > 0 ? pos[0] : "input.svg";
    const std::string solution = pos.size() > 1 ? pos[1] : "output.svg";
    const std::string stats = pos.size() > 2 ? pos[2] : "output.stats";
    const std::string config = pos.size() > 3 ? pos[3] : "config.cfg";
    std::printf("%s %s %s %s %s\n", argv[0], data.c_str(), solution.c_str(), stats.c_str(), config.c_str());

    int64_t n = 0;
    int dim = 0;
    emst_status st = emst_read_points(data.c_str(), nullptr, 0, &n, &dim);
    if (st != EMST_OK) return fail(nullptr, st, ("reading " + data).c_str());
    std::vector<float> pts((size_t)(n > 0 ? n : 1) * dim);
    if ((st = emst_read_points(data.c_str(), pts.data(), n, &n, &dim)) != EMST_OK)
        return fail(nullptr, st, ("reading " + data).c_str());

    emst_config cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.device = device;
    cfg.search_mode = static_table ? 1 : 0;
    emst_ctx* ctx = nullptr;
    if ((st = emst_create(&cfg, &ctx)) != EMST_OK) return fail(nullptr, st, "emst_create");
    std::vector<int32_t> uv((size_t)2 * (n > 1 ? n - 1 : 1));
    int64_t ne = 0;
    double length = 0.0;
    const auto t0 = std::chrono::steady_clock::now();
    if ((st = emst_solve(ctx, pts.data(), n, dim, uv.data(), &ne, &length)) != EMST_OK)
        return fail(ctx, st, "emst_solve");
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    int64_t rounds = 0;
    if ((st = emst_get_round_stats(ctx, &rounds, nullptr, 0)) != EMST_OK) return fail(ctx, st, "round stats");
    const std::string base = base_of(solution);
    if ((st = emst_write_results(ctx, base.c_str())) != EMST_OK) return fail(ctx, st, "writing results");
    if (FILE* f = std::fopen(stats.c_str(), "a")) {
        std::fprintf(f, "%lld %d %lld %.6f %lld %.3f %s\n", (long long)n, dim, (long long)ne, length, (long long)rounds, ms,
                     data.c_str());
        std::fclose(f);
    }
    std::printf("points %lld dim %d edges %lld length %.6f rounds %lld time %.3f ms -> %s.links\n", (long long)n, dim,
                (long long)ne, length, (long long)rounds, ms, base.c_str());
    emst_destroy(ctx);
    return 0;
}
