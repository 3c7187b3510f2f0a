// ibtfo_run: the reference time loop (Test/Sod/Sod.cpp:27-195,
// Test/InclineSod/InclineSod.cpp:30-204) on the GB300 library.
//
//   ibtfo_run case.inp [--case NAME] [--steps N] [--print-every K] [--out FILE]
//                      [--vtk [--vtk-every V] [--vtk-binary]] [--checkpoint FILE] [--restart FILE]
//
// Reads the .inp numbers exactly as the reference's ParamReader does, plus the
// slot keys Scheme / Riemann / Limiter / Boundary / Global_Boundary /
// Precision and `Case` (the plug-in: sod_ref, sod_x, incline_ref, vortex_ref,
// channel, isentropic_vortex).  Prints the reference's per-iteration line
// ("iter : N.   dt :X.   time :T.  Mass loss :M") every K iterations (every
// iteration by default, like the reference) and writes the final U_OLD
// (M*N*4 doubles, reference layout) to FILE.  --vtk writes dat_0_<iter>.vtk
// files listed in result.visit (Src/Utils/WriteData.cpp:20-27) when the
// reference's test drivers do (Test/Sod/Sod.cpp:135-152): before an iteration
// whose number is a multiple of the .inp's plot_per (default 100) when
// plot_int is 0, else before the first iteration and whenever the time has
// passed the next of plot_int equal fractions of Psy_time; and once after the
// loop.  --vtk-every V sets plot_per = V, plot_int = 0.  --checkpoint saves
// the final state to restart from; --restart continues from such a file
// instead of the initial state.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ibtfo.h"

static int die(const char *what)
{
    fprintf(stderr, "ibtfo_run: %s: %s\n", what, ibtfo_last_error());
    return 1;
}

int main(int argc, char **argv)
{
    if (argc < 2)
    {
        fprintf(stderr,
                "usage: %s case.inp [--case NAME] [--steps N] [--print-every K] [--out FILE] "
                "[--vtk [--vtk-every V] [--vtk-binary]] [--checkpoint FILE] [--restart FILE]\n",
                argv[0]);
        return 2;
    }
    const char *inp_path = argv[1];
    std::string case_name, out_path, ckpt_path, restart_path;
    long steps = -1, every = 1, vtk_every = 0;
    int vtk = 0, vtk_binary = 0;
    for (int a = 2; a < argc; a++)
    {
        std::string s = argv[a];
        if (s == "--case" && a + 1 < argc)
            case_name = argv[++a];
        else if (s == "--steps" && a + 1 < argc)
            steps = atol(argv[++a]);
        else if (s == "--print-every" && a + 1 < argc)
            every = std::max(1L, atol(argv[++a]));
        else if (s == "--out" && a + 1 < argc)
            out_path = argv[++a];
        else if (s == "--vtk")
            vtk = 1;
        else if (s == "--vtk-every" && a + 1 < argc)
            vtk = 1, vtk_every = atol(argv[++a]);
        else if (s == "--vtk-binary")
            vtk_binary = 1;
        else if (s == "--checkpoint" && a + 1 < argc)
            ckpt_path = argv[++a];
        else if (s == "--restart" && a + 1 < argc)
            restart_path = argv[++a];
        else
        {
            fprintf(stderr, "ibtfo_run: unknown argument %s\n", s.c_str());
            return 2;
        }
    }
    ibtfo_inp *inp = nullptr;
    if (ibtfo_inp_open(inp_path, &inp) != IBTFO_OK)
        return die("reading the .inp file");
    ibtfo_config cfg;
    if (ibtfo_config_from_inp(inp, &cfg) != IBTFO_OK)
        return die("configuration");
    if (case_name.empty())
    {
        char buf[128];
        case_name = (ibtfo_inp_get_string(inp, "Case", buf, sizeof buf) && buf[0]) ? buf : "sod_ref";
    }
    printf(" ==== parameters are read ====\n");
    const int M = cfg.n_x + 2 * cfg.num_ghost_cell, N = cfg.n_y + 2 * cfg.num_ghost_cell;
    std::vector<double> phi((size_t)M * N), xy((size_t)M * N * 6), u((size_t)M * N * 4);

    ibtfo_case *cs = nullptr;
    if (ibtfo_create(&cfg, &cs) != IBTFO_OK)
        return die("ibtfo_create");
    if (ibtfo_case_phi(case_name.c_str(), inp, &cfg, phi.data()) != IBTFO_OK)
        return die("level set plug-in");
    if (ibtfo_setup_geometry(cs, phi.data()) != IBTFO_OK || ibtfo_get_geometry(cs, xy.data()) != IBTFO_OK)
        return die("geometry");
    printf(" ====  Geometry Initialize complete ====\n");
    if (ibtfo_case_init(case_name.c_str(), inp, &cfg, xy.data(), u.data()) != IBTFO_OK)
        return die("initial-state plug-in");
    if (restart_path.empty() ? ibtfo_set_state(cs, u.data()) != IBTFO_OK
                             : ibtfo_load_checkpoint(cs, restart_path.c_str()) != IBTFO_OK)
        return die(restart_path.empty() ? "ibtfo_set_state" : "ibtfo_load_checkpoint");
    ibtfo_progress p;
    ibtfo_get_progress(cs, &p);
    printf(" ====  Initial Mass is %g ====\n", p.mass_start);
    auto write_vtk = [&](int iter) -> bool {
        const std::string name = "dat_0_" + std::to_string(iter) + ".vtk";
        FILE *visit = fopen("result.visit", "a");
        if (!visit)
            return false;
        if (iter == 0)
            fprintf(visit, "!NBLOCKS 1\n");
        fprintf(visit, "%s\n", name.c_str());
        fclose(visit);
        return ibtfo_write_vtk_async(cs, name.c_str(), vtk_binary) == IBTFO_OK;
    };
    double plot_per = 100, plot_int = 0;
    ibtfo_inp_get(inp, "plot_per", 100, &plot_per);
    ibtfo_inp_get(inp, "plot_int", 0, &plot_int);
    if (vtk_every > 0)
        plot_per = (double)vtk_every, plot_int = 0;
    const long per = std::max<long>(1, (long)plot_per);
    const int n_int = (int)plot_int;
    int output_int = 1;
    const long limit = steps >= 0 ? steps : cfg.max_iter;
    while (p.now_t < cfg.psy_time && p.iter < cfg.max_iter && p.iter < limit)
    {
        if (vtk)
        {
            const bool due = n_int == 0 ? p.iter % per == 0
                                        : (p.now_t > output_int * cfg.psy_time / n_int || p.iter == 0);
            if (due && !write_vtk(p.iter))
                return die("writing VTK");
            if (due && n_int != 0 && p.iter > 0)
                output_int++;
        }
        long n = std::min<long>(every - p.iter % every, limit - p.iter);
        if (vtk)
            n = n_int == 0 ? std::min<long>(n, per - p.iter % per) : 1; // the time rule looks at every iteration
        if (ibtfo_advance(cs, (int)n) != IBTFO_OK || ibtfo_get_progress(cs, &p) != IBTFO_OK)
            return die("stepping");
        if (p.iter % every == 0 || p.now_t >= cfg.psy_time || p.iter >= limit)
            printf("iter : %d.   dt :%g.   time :%g.  Mass loss :%g\n", p.iter, p.dt, p.now_t,
                   std::fabs(p.mass - p.mass_start));
    }
    if (vtk && (!write_vtk(p.iter) || ibtfo_output_wait(cs) != IBTFO_OK))
        return die("writing VTK");
    if (!ckpt_path.empty() && ibtfo_save_checkpoint(cs, ckpt_path.c_str()) != IBTFO_OK)
        return die("ibtfo_save_checkpoint");
    if (!out_path.empty())
    {
        if (ibtfo_get_state(cs, u.data(), nullptr) != IBTFO_OK)
            return die("ibtfo_get_state");
        FILE *f = fopen(out_path.c_str(), "wb");
        if (!f || fwrite(u.data(), sizeof(double), u.size(), f) != u.size())
        {
            fprintf(stderr, "ibtfo_run: cannot write %s\n", out_path.c_str());
            return 1;
        }
        fclose(f);
    }
    ibtfo_destroy(cs);
    ibtfo_inp_close(inp);
    return 0;
}
