// cli.cpp -- command-line driver with the reference's main() behaviour
// (src/main.cu:75-102): read ../inputs/inputs.txt, advance tmax steps, write
// ../results/{p,uc,vc,final_results}.dat.  Optional arguments override the
// inputs file and the results directory.
#include <cstdio>

#include "immerseflow_gb300.h"

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
    int steps = 0;
    while (steps < c.tmax) {
        if (ifx_step(s, 1) != IFX_OK) {
            std::fprintf(stderr, "step %d: %s\n", steps, ifx_last_error());
            rc = 1;
            break;
        }
        steps++;
    }
    ifx_stats st;
    if (ifx_get_stats(s, 0, &st) == IFX_OK)
        std::printf("steps %lld, last predictor sweeps %d, last pressure iterations %d, cd %.6f, cl %.6f\n",
                    st.steps, st.last_ad_iters, st.last_ppe_iters, st.cd, st.cl);
    if (ifx_write_results(s, results) != IFX_OK) {
        std::fprintf(stderr, "%s\n", ifx_last_error());
        rc = 1;
    }
    ifx_destroy(s);
    return rc;
}
