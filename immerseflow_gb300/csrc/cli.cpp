// cli.cpp -- command-line driver with the reference's main() behaviour
// (src/main.cu:75-102): read ../inputs/inputs.txt, advance tmax steps, write
// ../results/{p,uc,vc,final_results}.dat.  Optional arguments override the
// inputs file and the results directory.
//
// Restart and snapshots (parsed by the reference, src/main.cu:27-30,50-53, and
// used by its Fortran predecessor, test/UTIL_PRE_SIM.f90:120-149): every
// `Write Interval` steps the state is written to <results>/Data/data.NNNNNNN.ifx
// (binary, exact) and .dat (ASCII, predecessor layout), NNNNNNN = int(t); with
// Restart = 1 the run starts from data.<Restart_Time> (the binary file if
// present, else the ASCII one) and continues to tmax steps.
// Probes (METHOD mode): a probe.dat beside the inputs file selects probe
// points; the run writes <results>/probe_output.dat and <results>/forces.dat.
#include <sys/stat.h>

#include <cstdio>
#include <string>
#include <vector>

#include "immerseflow_gb300.h"

static bool exists(const std::string& p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

static std::string snapshot_base(const char* results, long long index) {
    char name[64];
    std::snprintf(name, sizeof(name), "/Data/data.%07lld", index);
    return std::string(results) + name;
}

int main(int argc, char** argv) {
    const char* inputs = argc > 1 ? argv[1] : "../inputs/inputs.txt";
    const char* results = argc > 2 ? argv[2] : "../results";
    ifx_config c;
    if (ifx_config_read(inputs, &c) != IFX_OK) {
        std::fprintf(stderr, "%s\n", ifx_last_error());
        return 1;
    }
    ifx_solver* s = nullptr;
    if (ifx_create_from_file(inputs, &s) != IFX_OK) {
        std::fprintf(stderr, "%s\n", ifx_last_error());
        return 1;
    }
    std::printf("%s: %dx%d cells, %s mode, %d steps\n", ifx_version(), c.nx, c.ny,
                c.mode == IFX_MODE_METHOD ? "method" : "reference", (int)c.tmax);
    int rc = 0;
    if (c.restart) {
        const std::string base = snapshot_base(results, c.restart_time);
        ifx_status st = exists(base + ".ifx") ? ifx_checkpoint_read(s, (base + ".ifx").c_str())
                                              : ifx_read_snapshot_ascii(s, 0, (base + ".dat").c_str());
        if (st != IFX_OK) {
            std::fprintf(stderr, "restart: %s\n", ifx_last_error());
            ifx_destroy(s);
            return 1;
        }
    }
    bool probes = false;
    if (c.mode == IFX_MODE_METHOD) {
        std::string dir(inputs);
        const size_t slash = dir.find_last_of('/');
        dir = slash == std::string::npos ? std::string(".") : dir.substr(0, slash);
        const std::string pf = dir + "/probe.dat";
        std::vector<double> xy;
        int n = 0;
        if (exists(pf) && ifx_probes_read(pf.c_str(), 0, nullptr, &n) == IFX_OK && n > 0) {
            xy.resize(2 * (size_t)n);
            probes = ifx_probes_read(pf.c_str(), n, xy.data(), &n) == IFX_OK;
        }
        const int cap = c.tmax > 1e6 ? 1000000 : (int)c.tmax + 1;
        if (ifx_set_history(s, 0, cap, probes ? n : 0, probes ? xy.data() : nullptr) != IFX_OK) {
            std::fprintf(stderr, "history: %s\n", ifx_last_error());
            rc = 1;
        }
    }
    ifx_stats st0;
    long long steps = ifx_get_stats(s, 0, &st0) == IFX_OK ? st0.steps : 0;
    if (c.write_interval > 0) mkdir((std::string(results) + "/Data").c_str(), 0755);
    while (rc == 0 && steps < c.tmax) {
        if (ifx_step(s, 1) != IFX_OK) {
            std::fprintf(stderr, "step %lld: %s\n", steps, ifx_last_error());
            rc = 1;
            break;
        }
        steps++;
        if (c.write_interval > 0 && steps % c.write_interval == 0) {
            const std::string base = snapshot_base(results, (long long)(steps * c.dt));
            if (ifx_checkpoint_write(s, (base + ".ifx").c_str()) != IFX_OK ||
                ifx_write_snapshot_ascii(s, 0, (base + ".dat").c_str()) != IFX_OK) {
                std::fprintf(stderr, "snapshot: %s\n", ifx_last_error());
                rc = 1;
            }
        }
    }
    ifx_stats st;
    if (ifx_get_stats(s, 0, &st) == IFX_OK)
        std::printf("steps %lld, last predictor sweeps %d, last pressure iterations %d, cd %.6f, cl %.6f\n",
                    st.steps, st.last_ad_iters, st.last_ppe_iters, st.cd, st.cl);
    if (ifx_write_results(s, results) != IFX_OK) {
        std::fprintf(stderr, "%s\n", ifx_last_error());
        rc = 1;
    }
    if (c.mode == IFX_MODE_METHOD) {
        const std::string r(results);
        if ((probes && ifx_write_probe_file(s, 0, (r + "/probe_output.dat").c_str()) != IFX_OK) ||
            ifx_write_force_file(s, 0, (r + "/forces.dat").c_str()) != IFX_OK) {
            std::fprintf(stderr, "%s\n", ifx_last_error());
            rc = 1;
        }
    }
    ifx_destroy(s);
    return rc;
}
