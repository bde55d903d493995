// Tuned build schedules (no reference counterpart: the reference's superstep
// size is the fixed label budget -s, shared_memory/hhl.cpp:65).
//
// plant_gb300/autotune.py times candidate schedules on the GPU and writes the
// winners as a table, one graph class per line:
//     <class> first_superstep growth sf queue_split window_target window_warps ps
// A build with opts.autotune set takes, for every schedule option it leaves
// at 0 (auto), the value of its graph's class from that table: the file named
// by $CHL_SCHEDULES, else tuned_schedules.txt next to this library.  The
// class is the one autotune.graph_key computes: directedness, log2 n, the
// mean out-degree and whether the largest out-degree exceeds 32 times the
// mean.  Lines starting with '#' are comments.  A missing file or class
// leaves the built-in defaults.
#include "chl_internal.h"

#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

namespace chl {

std::string graph_class(const chl_graph *g) {
    const uint32_t n = g->n ? g->n : 1;
    uint64_t maxdeg = 0;
    for (uint32_t v = 0; v < g->n; ++v) maxdeg = std::max<uint64_t>(maxdeg, g->off[1][v + 1] - g->off[1][v]);
    const double mean = g->n ? (double)g->off[1][g->n] / g->n : 0.0;
    const double skew = mean > 0 ? (double)maxdeg / mean : 0.0;
    char buf[96];
    // round half to even, as Python's round()
    snprintf(buf, sizeof(buf), "%s-n2^%d-deg%d-skew%s", g->symmetric ? "sym" : "dir",
             (int)std::nearbyint(std::log2((double)n)), (int)std::nearbyint(mean), skew > 32 ? "heavy" : "flat");
    return buf;
}

static std::string table_path() {
    const char *env = getenv("CHL_SCHEDULES");
    if (env && *env) return env;
    Dl_info info;
    if (dladdr((void *)&table_path, &info) && info.dli_fname) {
        std::string p = info.dli_fname;
        const size_t slash = p.rfind('/');
        return (slash == std::string::npos ? std::string(".") : p.substr(0, slash)) + "/tuned_schedules.txt";
    }
    return "tuned_schedules.txt";
}

bool apply_tuned_schedule(const chl_graph *g, chl_build_opts &o) {
    FILE *f = fopen(table_path().c_str(), "r");
    if (!f) return false;
    const std::string cls = graph_class(g);
    char line[512], name[128];
    bool found = false;
    while (!found && fgets(line, sizeof(line), f)) {
        if (line[0] == '#') continue;
        unsigned first = 0, wt = 0, ww = 0;
        double growth = 0, sf = 0, ps = 0;
        int qs = 0;
        if (sscanf(line, "%127s %u %lf %lf %d %u %u %lf", name, &first, &growth, &sf, &qs, &wt, &ww, &ps) != 8)
            continue;
        if (cls != name) continue;
        found = true;
        if (!o.first_superstep) o.first_superstep = first;
        if (o.growth <= 0) o.growth = growth;
        if (o.sf <= 0) o.sf = sf;
        if (!o.queue_split) o.queue_split = qs;
        if (!o.window_target) o.window_target = wt;
        if (!o.window_warps) o.window_warps = ww;
        if (o.ps <= 0) o.ps = ps;
    }
    fclose(f);
    return found;
}

}  // namespace chl

extern "C" int chl_graph_class(const chl_graph *g, char *buf, size_t cap) {
    if (!g || !buf || cap == 0) return CHL_ERR_INVALID;
    const std::string c = chl::graph_class(g);
    if (c.size() + 1 > cap) return CHL_ERR_INVALID;
    memcpy(buf, c.c_str(), c.size() + 1);
    return CHL_OK;
}
