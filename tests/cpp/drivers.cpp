// drivers.cpp -- two reference host programs rewritten against include/lqt.h
// only (no Python): the way a maintainer of the reference would call the
// library from C++.
//
//   drivers oned   <out.dat>                         OneD.cc: 100-cell strand,
//        S1 every 1000 ms for 6 s, V of every cell every 10 steps in the
//        VentOneDResults layout; prints the conduction velocity.
//   drivers tissue <geometry.txt> <stim.cnd> <nx> <ny> <nz> <steps> <outdir>
//        GPU3D.cu: geometry and stimulation profile in the reference's text
//        formats, mixed-form tissue run with a VTK frame every 500 steps
//        (asynchronous writer) and V of every tissue voxel at the end in
//        <outdir>/v_final.bin.
//   drivers single <out.dat> <states.dat> <steps>    SingleCell.cc: one M cell
//        through the Cell interface (setIstim, update, getV, getICaL, getIKs,
//        getAbsDvdt), S1 -53 pA/pF x 1 ms at 50 ms of each 1000 ms cycle;
//        rows "time V ICaL IKs" every step; the final state dumped with
//        outputAllStates, read back with readinAllStates into a second cell
//        and checked; prints the largest |dV/dt| seen.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "lqt.h"

#define CHECK(call)                                                                           \
    do {                                                                                      \
        int rc_ = (call);                                                                     \
        if (rc_ != LQT_OK) {                                                                  \
            std::fprintf(stderr, "%s failed (%d): %s\n", #call, rc_, lqt_last_error());      \
            return 1;                                                                         \
        }                                                                                     \
    } while (0)

static int oned(const char *out)
{
    // OneD.cc:46-83: 25 endo, 35 M, 40 epi; dx 0.15; BCL 1000; 5 S1 + 1 cycle
    std::vector<uint8_t> types;
    for (int i = 0; i < 100; ++i) types.push_back(i < 25 ? LQT_ENDO : (i < 60 ? LQT_MCELL : LQT_EPI));
    lqt_model m;
    CHECK(lqt_model_preset(LQT_PRESET_CPU_DEFAULT, &m));
    lqt_instance inst;
    std::memset(&inst, 0, sizeof(inst));
    inst.ncells = 100;
    inst.n_stim = 3;
    inst.record = 1;
    inst.dx = 0.15;
    inst.bcl = 1000.0;
    inst.s1_start = 50.0;
    inst.s1_duration = 1.0;
    inst.s1_strength = -52.0;
    inst.t_stop = 6000.0;
    inst.ecg_x0 = 35.0;
    inst.act_threshold = -30.0;
    lqt_batch_params p;
    std::memset(&p, 0, sizeof(p));
    p.dt = 0.02;
    p.v0 = -87.5;
    p.precision = LQT_FP64;
    p.max_beats = 8;
    p.rec_every = 10;
    lqt_batch *b = nullptr;
    CHECK(lqt_batch_create(&p, 1, &inst, types.data(), nullptr, 1, &m, &b));
    CHECK(lqt_batch_run(b));
    int64_t nrec = 0;
    CHECK(lqt_batch_get_record(b, 0, nullptr, nullptr, nullptr, 0, &nrec));
    std::vector<double> v((size_t)nrec * 100), t((size_t)nrec), rows((size_t)nrec * 101);
    CHECK(lqt_batch_get_record(b, 0, v.data(), t.data(), nullptr, nrec, &nrec));
    for (int64_t r = 0; r < nrec; ++r) {
        rows[r * 101] = t[r];
        std::memcpy(&rows[r * 101 + 1], &v[r * 100], 100 * sizeof(double));
    }
    CHECK(lqt_io_write_dat(out, nrec, 101, rows.data(), 0));
    // CV between cells 10 and 90 on the last S1 cycle (OneD.cc:419-444)
    std::vector<float> tact(100 * 8);
    CHECK(lqt_batch_get_detect(b, tact.data(), nullptr, nullptr, nullptr, nullptr));
    double s = -1, e = -1;
    for (int k = 0; k < 8; ++k) {
        if (tact[10 * 8 + k] >= 5000 && tact[10 * 8 + k] < 6000 && s < 0) s = tact[10 * 8 + k];
        if (tact[90 * 8 + k] >= 5000 && tact[90 * 8 + k] < 6000 && e < 0) e = tact[90 * 8 + k];
    }
    std::printf("cv %.6f\n", (s >= 0 && e >= 0) ? 0.15 * 80 / (e - s) : -1.0);
    lqt_batch_destroy(b);
    return 0;
}

static int tissue(const char *geom_path, const char *stim_path, int nx, int ny, int nz, long steps, const char *outdir)
{
    const size_t ng = (size_t)nx * ny * nz;
    std::vector<uint8_t> types(ng), code(ng), s2(ng), s1(ng);
    std::vector<float> fibre(ng * 3), onset(ng);
    lqt_geom_file_spec gs = {3, nx, ny, nz, 0, 0};
    int64_t ntissue = 0, npts = 0;
    CHECK(lqt_io_read_geometry(geom_path, &gs, types.data(), code.data(), fibre.data(), s2.data(), &ntissue));
    CHECK(lqt_io_read_stimulation(stim_path, nx, ny, nz, -1, types.data(), s1.data(), onset.data(), &npts));
    lqt_model m;
    CHECK(lqt_model_preset(LQT_PRESET_LQT1, &m));
    lqt_geometry g = {nx, ny, nz, 0.2, types.data(), fibre.data(), 0.154, 0.0385, nullptr};
    lqt_sim_params sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.dt = 0.02;
    sp.v0 = -87.5;
    sp.precision = LQT_MIXED;
    sp.detect = 1;
    sp.model = m;
    sp.act_threshold = -30.0;
    sp.vmin_ok = -200.0;
    sp.vmax_ok = 200.0;
    lqt_sim *s = nullptr;
    CHECK(lqt_sim_create(&sp, &g, &s));
    lqt_protocol q;
    std::memset(&q, 0, sizeof(q));
    q.bcl = 500.0;          // BCL1 of GPU3D.cu:1726
    q.s1_start = 0.0;
    q.s1_duration = 2.0;
    q.s1_strength = -52.0;
    q.s1_mask = s1.data();
    q.s1_onset = onset.data();
    q.s2_time = -1.0;
    CHECK(lqt_sim_set_protocol(s, &q));
    lqt_vtk_writer *w = nullptr;
    CHECK(lqt_vtk_writer_create(s, 3, 2, &w));
    for (long k = 0; k < steps; k += 500) {
        char name[512];
        std::snprintf(name, sizeof(name), "%s/ap_%ld.vtk", outdir, k / 50);
        CHECK(lqt_vtk_writer_submit(w, name));
        CHECK(lqt_sim_step(s, steps - k < 500 ? steps - k : 500));
    }
    CHECK(lqt_vtk_writer_flush(w));
    lqt_vtk_writer_destroy(w);
    int64_t bad = 0;
    CHECK(lqt_sim_check(s, &bad));
    const int64_t n = lqt_sim_num_tissue(s);
    std::vector<double> v((size_t)n);
    CHECK(lqt_sim_get_v(s, v.data(), 1));
    std::string path = std::string(outdir) + "/v_final.bin";
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(v.data(), sizeof(double), (size_t)n, f) != (size_t)n) return 1;
    std::fclose(f);
    std::printf("tissue %lld stimulated %lld steps %ld\n", (long long)ntissue, (long long)npts, steps);
    lqt_sim_destroy(s);
    return 0;
}

static int single(const char *out, const char *states, long steps)
{
    // SingleCell.cc:45-51: BCL 1000, dt 0.02, -53 pA/pF x 1 ms at 50 ms
    const double bcl = 1000.0, dt = 0.02, start = 50.0, dur = 1.0, strength = -53.0;
    const uint8_t mcell = LQT_MCELL;
    lqt_model m;
    CHECK(lqt_model_preset(LQT_PRESET_CPU_DEFAULT, &m));
    lqt_cells *c = nullptr;
    CHECK(lqt_cells_create(1, &mcell, LQT_FP64, &m, dt, nullptr, &c));
    FILE *f = std::fopen(out, "w");
    if (!f) return 1;
    double time = 0.0, dvdt_max = 0.0;
    for (long step = 0; step < steps; ++step, time += dt) {
        const double tb = time - std::floor(time / bcl) * bcl;
        const double ist = (tb >= start && tb < start + dur) ? strength : 0.0;
        CHECK(lqt_cells_set_inputs(c, &ist, nullptr));
        CHECK(lqt_cells_update(c, 1));
        double v, cur[6];
        CHECK(lqt_cells_get_v(c, &v));
        CHECK(lqt_cells_get_currents(c, cur));
        if (cur[5] > dvdt_max) dvdt_max = cur[5];
        std::fprintf(f, "%4.10f\t%4.10f\t%4.10f\t%4.10f\t\n", time, v, cur[1], cur[3]);
    }
    std::fclose(f);
    // outputAllStates / readinAllStates round trip through a file
    FILE *sf = std::fopen(states, "w");
    if (!sf) return 1;
    CHECK(lqt_cells_output_states(c, 0, 1, sf));
    std::fclose(sf);
    lqt_cells *c2 = nullptr;
    CHECK(lqt_cells_create(1, &mcell, LQT_FP64, &m, dt, nullptr, &c2));
    sf = std::fopen(states, "r");
    if (!sf) return 1;
    CHECK(lqt_cells_readin_states(c2, 0, 1, sf));
    std::fclose(sf);
    double a[LQT_NSTATE], b[LQT_NSTATE];
    CHECK(lqt_cells_get_state(c, a));
    CHECK(lqt_cells_get_state(c2, b));
    double worst = 0.0;
    for (int i = 0; i < LQT_NSTATE; ++i) worst = std::fmax(worst, std::fabs(a[i] - b[i]));
    std::printf("dvdt_max %.6f readin_max_diff %.3g\n", dvdt_max, worst);
    lqt_cells_destroy(c2);
    lqt_cells_destroy(c);
    return worst <= 5.1e-11 ? 0 : 3;
}

int main(int argc, char **argv)
{
    if (argc >= 3 && !std::strcmp(argv[1], "oned")) return oned(argv[2]);
    if (argc >= 5 && !std::strcmp(argv[1], "single")) return single(argv[2], argv[3], std::atol(argv[4]));
    if (argc >= 9 && !std::strcmp(argv[1], "tissue"))
        return tissue(argv[2], argv[3], std::atoi(argv[4]), std::atoi(argv[5]), std::atoi(argv[6]), std::atol(argv[7]),
                      argv[8]);
    std::fprintf(stderr, "usage: drivers oned <out.dat> | single <out.dat> <states.dat> <steps> | "
                         "tissue <geom> <stim> <nx> <ny> <nz> <steps> <outdir>\n");
    return 2;
}
