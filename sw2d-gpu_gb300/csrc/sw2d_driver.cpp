// sw2d_driver.cpp -- host driver with the reference's input/output surface.
//
// The reference SW2D-GPU (SW2D-GPU_linux/src/SW2D-GPU.cu, "cu:<line>") is a
// single main() that reads a fixed directory layout, runs its solver loop
// and writes VTK rasters, a probe time series and a timing file.  This
// program reads and writes the same files and runs the loop through the C
// ABI of libsw2d.so (include/sw2d.h):
//
//   db/dir.txt                          list of cases            (cu:772-776)
//   db/<case>/input/setup.dat           run settings             (cu:779-805)
//   db/<case>/input/dem.txt             ESRI ASCII DEM           (cu:815-835)
//   db/<case>/input/coord_source_sink.dat, Q_source_sink.dat     (cu:840-921)
//   db/<case>/input/rain.dat            rain series              (cu:929-960)
//   db/<case>/input/temperatures.txt, solar_radiation.txt        (cu:963-1016)
//   db/<case>/input/initial_condition.txt                        (cu:1022-1033)
//   db/<case>/input/coord_out.dat       probes                   (cu:1047-1069)
//   db/<case>/output/Results_<k>.vtk    depth, velocities, DEM   (cu:1339-1472)
//   db/<case>/output/WaterLevel.txt     probe depths             (cu:1386-1410)
//   db/<case>/output/TimeSimu_<k>.txt   run time                 (cu:1477-1485)
//
// Extensions, off unless asked for, so the reference's datasets give the
// reference's outputs:
//   db/<case>/input/manning.txt         per-cell Manning n, ESRI ASCII of the
//                                       DEM's shape (used when present; the
//                                       reference has one scalar, cu:799)
//   db/<case>/input/rain_weights.txt    spatial rain distribution: per-cell
//                                       factors of rain.dat's rate, ESRI ASCII
//                                       (used when present; the reference
//                                       rains one value everywhere, cu:654)
//   db/<case>/output/Outflow.txt        outflow hydrograph of the open south
//                                       edge (--south-open): time, cumulative
//                                       volume, mean rate since the last line
//
// Usage: sw2d_run [--db DIR] [--precision f64|f32] [--cfl C] [--south-open] [--max-outputs N]
//   --precision f64 (default) runs the reference's scheme with its fixed dt;
//   --cfl C switches to the CFL rule; --south-open opens the south edge (free
//   outfall); --max-outputs stops after N VTK files.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "sw2d.h"

namespace {

struct Setup {
    double t0[4] = {0, 0, 0, 0}, t1[4] = {0, 0, 0, 0};
    double dt = 0, dpout = 0, dkout = 0, dtoq = 0;
    int evaporation_on = 0;
    double EV_WL_min = 0, INT = 0, INF = 0, LWL = 0, manning = 0;
    int out_vx = 1, out_vy = 1, out_z = 1, out_h = 1, out_outlet = 0;
};

std::vector<std::string> tokens(const std::string &path) {
    std::ifstream f(path);
    std::vector<std::string> t;
    std::string w;
    while (f >> w) t.push_back(w);
    return t;
}

bool file_exists(const std::string &p) {
    std::ifstream f(p);
    return f.good();
}

// "key: v1 v2 ..." lines (cu:788-804); unknown keys are ignored, as the
// reference ignores trailing keys
bool read_setup(const std::string &path, Setup &s) {
    std::ifstream f(path);
    if (!f) return false;
    std::map<std::string, std::vector<double>> kv;
    std::string line;
    while (std::getline(f, line)) {
        const size_t c = line.find(':');
        if (c == std::string::npos) continue;
        std::string key = line.substr(0, c);
        key.erase(0, key.find_first_not_of(" \t\r"));
        key.erase(key.find_last_not_of(" \t\r") + 1);
        std::istringstream vs(line.substr(c + 1));
        std::vector<double> v;
        double x;
        while (vs >> x) v.push_back(x);
        kv[key] = v;
    }
    auto get = [&](const char *k, double def) { return kv.count(k) && !kv[k].empty() ? kv[k][0] : def; };
    if (kv.count("tday0_thour0_tmin0_tsec0"))
        for (int i = 0; i < 4 && i < (int)kv["tday0_thour0_tmin0_tsec0"].size(); i++)
            s.t0[i] = kv["tday0_thour0_tmin0_tsec0"][i];
    if (kv.count("tday_thour_tmin_tsec"))
        for (int i = 0; i < 4 && i < (int)kv["tday_thour_tmin_tsec"].size(); i++) s.t1[i] = kv["tday_thour_tmin_tsec"][i];
    s.dt = get("dt", 0);
    s.dpout = get("dpout", 0);
    s.dkout = get("dkout", 0);
    s.dtoq = get("dtoq", 1);
    s.evaporation_on = (int)get("evaporation_on", 0);
    s.EV_WL_min = get("EV_WL_min", 0);
    s.INT = get("INT", 0);
    s.INF = get("INF", 0);
    s.LWL = get("LWL", 0);
    s.manning = get("manning_coef", 0);
    s.out_vx = (int)get("out_velocity_x", 1);
    s.out_vy = (int)get("out_velocity_y", 1);
    s.out_z = (int)get("out_elevation", 1);
    s.out_h = (int)get("out_depth", 1);
    s.out_outlet = (int)get("out_outlet_on", 0);
    return s.dt > 0;
}

struct Esri {
    int cols = 0, rows = 0;
    double xll = 0, yll = 0, cell = 1, nodata = -9999;
    std::vector<double> v;
};

// ESRI ASCII grid: six "key value" header lines, then rows*cols values,
// north row first (cu:822-834)
bool read_esri(const std::string &path, Esri &g) {
    std::vector<std::string> t = tokens(path);
    size_t k = 0;
    std::map<std::string, double> hdr;
    while (k + 1 < t.size()) {
        char *end = nullptr;
        std::strtod(t[k].c_str(), &end);
        if (end && *end == '\0') break;  // first number: data starts
        std::string key = t[k];
        for (char &c : key) c = (char)std::tolower((unsigned char)c);
        hdr[key] = std::atof(t[k + 1].c_str());
        k += 2;
    }
    g.cols = (int)hdr["ncols"];
    g.rows = (int)hdr["nrows"];
    g.xll = hdr["xllcorner"];
    g.yll = hdr["yllcorner"];
    g.cell = hdr["cellsize"];
    g.nodata = hdr.count("nodata_value") ? hdr["nodata_value"] : -9999.0;
    const size_t n = (size_t)g.rows * g.cols;
    if (g.rows < 1 || g.cols < 1 || t.size() < k + n) return false;
    g.v.resize(n);
    for (size_t i = 0; i < n; i++) g.v[i] = std::atof(t[k + i].c_str());
    return true;
}

std::vector<double> read_numbers(const std::string &path, size_t skip_tokens = 0) {
    std::vector<std::string> t = tokens(path);
    std::vector<double> v;
    for (size_t i = skip_tokens; i < t.size(); i++) v.push_back(std::atof(t[i].c_str()));
    return v;
}

// "nst N" / "n_out N" followed by N coordinate pairs [m]
std::vector<std::pair<double, double>> read_coords(const std::string &path) {
    std::vector<std::string> t = tokens(path);
    std::vector<std::pair<double, double>> out;
    if (t.size() < 2) return out;
    const int n = std::atoi(t[1].c_str());
    for (int i = 0; i < n && 2 + 2 * i + 1 < (int)t.size(); i++)
        out.push_back({std::atof(t[2 + 2 * i].c_str()), std::atof(t[3 + 2 * i].c_str())});
    return out;
}

double c_round(double x) { return std::round(x); }  // half away from zero, as C round()

int check(sw2d_handle *h, int st, const char *what) {
    if (st != SW2D_OK) {
        std::fprintf(stderr, "%s failed: %s (%s)\n", what, sw2d_status_string(st), h ? sw2d_last_error(h) : "");
        std::exit(2);
    }
    return st;
}

struct Opts {
    std::string db = "db";
    int precision = SW2D_PREC_F64;
    double cfl = 0.0;
    bool south_open = false;
    long max_outputs = -1;
};

int run_case(const Opts &o, const std::string &name) {
    const std::string in = o.db + "/" + name + "/input/", out = o.db + "/" + name + "/output/";
    Setup su;
    if (!read_setup(in + "setup.dat", su)) {
        std::printf("unknown file - setup.dat\n");
        return 1;
    }
    Esri dem;
    if (!read_esri(in + "dem.txt", dem)) {
        std::printf("unknown file - dem.txt\n");
        return 1;
    }
    const int rows = dem.rows, cols = dem.cols;
    const double res = dem.cell;
    const size_t ncell = (size_t)rows * cols;
    // sources: coordinates in m -> cells; the reference's linear index
    // (cu:542-545, Linux); an index past the grid lands in its padding row
    // and has no effect there, so it is dropped here
    std::vector<std::pair<double, double>> src = read_coords(in + "coord_source_sink.dat");
    std::vector<double> qraw = read_numbers(in + "Q_source_sink.dat", 2);  // "flow (m3/s)"
    const int nst = (int)src.size();
    std::vector<int32_t> cells;
    std::vector<int> keep;
    for (int i = 0; i < nst; i++) {
        const long qinx = (long)c_round(std::fabs(dem.xll / res - src[i].first / res));
        const long qiny = rows - (long)c_round(std::fabs(dem.yll / res - src[i].second / res));
        const long idx = (qiny + 1) * cols - (cols - (qinx + 1));
        if (idx >= 0 && idx < (long)ncell) {
            cells.push_back((int32_t)idx);
            keep.push_back(i);
        }
    }
    const int nrec = nst > 0 ? (int)(qraw.size() / nst) : 0;
    std::vector<double> q((size_t)nrec * keep.size());
    for (int r = 0; r < nrec; r++)
        for (size_t k = 0; k < keep.size(); k++) q[(size_t)r * keep.size() + k] = qraw[(size_t)r * nst + keep[k]];
    // rain: dtrain, a 4-token header, then "time value" pairs (cu:952-959)
    std::vector<std::string> rt = tokens(in + "rain.dat");
    if (rt.size() < 5) {
        std::printf("unknown file - rain.dat\n");
        return 1;
    }
    const double dtrain = std::atof(rt[0].c_str());
    std::vector<double> rain;
    for (size_t i = 5 + 1; i < rt.size(); i += 2) rain.push_back(std::atof(rt[i].c_str()));
    // evaporation (cu:963-1016, cu:1242-1245)
    std::vector<double> evapo;
    if (su.evaporation_on == 1) {
        std::vector<std::string> sr = tokens(in + "solar_radiation.txt");
        std::vector<double> T = read_numbers(in + "temperatures.txt", 1);
        if (sr.size() < 3 || T.empty()) {
            std::printf("unknown file - evaporation.dat\n");
            return 1;
        }
        const double albedo = std::atof(sr[1].c_str());
        std::vector<double> Rg;
        for (size_t i = 3; i < sr.size(); i++) Rg.push_back(std::atof(sr[i].c_str()));
        const size_t n = std::min(T.size(), Rg.size());
        T.resize(n);
        Rg.resize(n);
        evapo.resize(n);
        if (sw2d_evaporation_series(T.data(), Rg.data(), (int32_t)n, albedo, dtrain, evapo.data()) != SW2D_OK) {
            std::printf("unknown file - evaporation.dat\n");
            return 1;
        }
    }
    // optional roughness raster (extension)
    Esri nman;
    const bool has_n = file_exists(in + "manning.txt");
    if (has_n && (!read_esri(in + "manning.txt", nman) || nman.rows != rows || nman.cols != cols)) {
        std::printf("unknown file - manning.txt\n");
        return 1;
    }
    Esri rainw;
    const bool has_w = file_exists(in + "rain_weights.txt");
    if (has_w && (!read_esri(in + "rain_weights.txt", rainw) || rainw.rows != rows || rainw.cols != cols)) {
        std::printf("unknown file - rain_weights.txt\n");
        return 1;
    }
    std::vector<double> ic = read_numbers(in + "initial_condition.txt");
    if (ic.size() < ncell) {
        std::printf("unknown file - initial_condition.txt\n");
        return 1;
    }
    ic.resize(ncell);
    // probes (cu:1047-1069)
    std::vector<std::pair<double, double>> probes;
    if (su.out_outlet == 1) {
        if (!file_exists(in + "coord_out.dat")) {
            std::printf("unknown file - coord_out.dat\n");
            return 1;
        }
        probes = read_coords(in + "coord_out.dat");
    }
    const long lpout = std::lround(su.dpout / su.dt), lkout = std::lround(su.dkout / su.dt);  // cu:1039-1040
    const double time0 = 3600.0 * 24.0 * su.t0[0] + 3600.0 * su.t0[1] + 60.0 * su.t0[2] + su.t0[3];
    double timmax = 3600.0 * 24.0 * su.t1[0] + 3600.0 * su.t1[1] + 60.0 * su.t1[2] + su.t1[3];
    if (su.t1[0] == 0 && su.t1[1] == 0 && su.t1[2] == 0 && su.t1[3] == 0) {
        // (cont_rain - 2) * dtrain with cont_rain = newline characters of rain.dat (cu:939-946, cu:1085-1087)
        std::ifstream rf(in + "rain.dat", std::ios::binary);
        long nl = 0;
        for (char c; rf.get(c);)
            if (c == '\n') nl++;
        timmax = (double)(nl - 2) * dtrain;
    }

    sw2d_config cfg;
    sw2d_config_init(&cfg);
    cfg.rows = rows;
    cfg.cols = cols;
    cfg.dx = cfg.dy = res;
    cfg.nodata = dem.nodata;
    cfg.manning = su.manning;
    cfg.INT = su.INT;
    cfg.INF = su.INF;
    cfg.LWL = su.LWL;
    cfg.EV_WL_min = su.EV_WL_min;
    cfg.precision = o.precision;
    cfg.dt = su.dt;
    if (o.cfl > 0) {
        cfg.dt_mode = SW2D_DT_CFL;
        cfg.cfl = o.cfl;
    }
    cfg.south_open = o.south_open ? 1 : 0;
    sw2d_handle *h = nullptr;
    check(nullptr, sw2d_create(&cfg, &h), "sw2d_create");
    check(h, sw2d_set_static(h, dem.v.data(), has_n ? nman.v.data() : nullptr), "sw2d_set_static");
    if (has_w) check(h, sw2d_set_rain_weights(h, rainw.v.data()), "sw2d_set_rain_weights");
    check(h, sw2d_set_state(h, ic.data(), nullptr, nullptr, time0), "sw2d_set_state");
    check(h, sw2d_set_rain(h, SW2D_RAIN_COMPAT, rain.data(), (int32_t)rain.size(), dtrain), "sw2d_set_rain");
    if (!evapo.empty())
        check(h, sw2d_set_evaporation(h, evapo.data(), (int32_t)evapo.size(), dtrain), "sw2d_set_evaporation");
    if (!cells.empty() && nrec > 0)
        check(h, sw2d_set_point_sources(h, cells.data(), (int32_t)cells.size(), q.data(), nrec, su.dtoq),
              "sw2d_set_point_sources");

    std::printf("%s\n", " ********************************************************************");
    std::printf("%s\n", " Two-dimensional shallow water model, GB300 time-stepping core (sw2d)");
    std::printf("%s\n", " ********************************************************************");
    std::printf("%s\n", name.c_str());

    FILE *wl = std::fopen((out + "WaterLevel.txt").c_str(), "w");
    if (!wl) {
        std::printf("cannot write %sWaterLevel.txt\n", out.c_str());
        return 1;
    }
    if (su.out_outlet != 1) std::fprintf(wl, "%s\n", "Outlet off");
    FILE *hyd = nullptr;  // outflow hydrograph (extension)
    double hyd_t = time0, hyd_v = 0.0;
    if (o.south_open) {
        hyd = std::fopen((out + "Outflow.txt").c_str(), "w");
        if (!hyd) {
            std::printf("cannot write %sOutflow.txt\n", out.c_str());
            return 1;
        }
        std::fprintf(hyd, "%s\n", "time_s outflow_volume_m3 outflow_rate_m3_per_s");
    }
    // probe cells in the row-major order the reference visits them (cu:1388-1410)
    std::vector<long> probe_km;
    for (auto &p : probes) {
        const long outx = (long)c_round(std::fabs(dem.xll / res - p.first / res));
        const long outy = rows - (long)c_round(std::fabs(dem.yll / res - p.second / res));
        probe_km.push_back(outy * cols - (cols - (outx + 1)));
    }

    std::vector<double> hh(ncell), uu(ncell), vv(ncell);
    const auto t_start = std::chrono::steady_clock::now();
    long iters = 0, mstep = 0, outputs = 0;
    std::string tempo = "0";
    // outputs come after the first iteration and then whenever mstep (two
    // per iteration) is a multiple of lkout (cu:1339)
    const long per_out = lkout > 0 ? (lkout % 2 == 0 ? lkout / 2 : lkout) : 1;
    bool first = true;
    for (;;) {
        const long chunk = first ? 1 : per_out - (iters % per_out);
        int64_t done = 0;
        check(h, sw2d_advance(h, chunk, timmax, &done), "sw2d_advance");
        if (done == 0) break;
        for (long k = 0; k < done; k++) {  // progress line at the start of an iteration (cu:1260-1262)
            const long m = mstep + 2 * k;
            if (lpout > 0 && m % lpout == 0) std::printf(" %d\n", (int)(time0 + (double)m * su.dt));
        }
        iters += done;
        mstep += 2 * done;
        if (!(first || (lkout > 0 && mstep % lkout == 0))) continue;
        tempo = first ? "0" : std::to_string((long long)c_round((double)mstep * su.dt / su.dkout));
        check(h, sw2d_get_field(h, SW2D_FIELD_DEPTH, hh.data()), "sw2d_get_field");
        FILE *vtk = std::fopen((out + "Results_" + tempo + ".vtk").c_str(), "w");
        if (!vtk) {
            std::printf("cannot write VTK output\n");
            return 1;
        }
        std::fprintf(vtk, "%s\n", "# vtk DataFile Version 2.0");
        std::fprintf(vtk, "%s\n", "Brazil");
        std::fprintf(vtk, "%s\n", "ASCII");
        std::fprintf(vtk, "%s\n", "DATASET STRUCTURED_POINTS");
        std::fprintf(vtk, "DIMENSIONS %d %d %d\n", cols, rows, 1);
        std::fprintf(vtk, "ASPECT_RATIO %lf %lf %lf\n", res, res, 1.0000);
        std::fprintf(vtk, "ORIGIN %lf %lf %lf\n", dem.xll, dem.yll, 0.000);
        std::fprintf(vtk, "POINT_DATA %d\n", cols * rows);
        // rows are written south first: VTK row 0 is the grid's last row (cu:1381)
        auto write_field = [&](const char *label, const std::vector<double> &f, double sign) {
            std::fprintf(vtk, "SCALARS %s float 1\n", label);
            std::fprintf(vtk, "%s\n", "LOOKUP_TABLE default");
            for (int im = 0; im < rows; im++) {
                const size_t base = (size_t)(rows - 1 - im) * cols;
                for (int jm = 0; jm < cols; jm++) {
                    const double v = f[base + jm];
                    std::fprintf(vtk, "%f\n", sign < 0 ? -v : v);
                }
            }
        };
        const std::vector<double> &depth = first ? ic : hh;  // cu:1415-1420
        if (su.out_h == 1) write_field("depth", depth, 1.0);
        if (su.out_vx == 1) {
            check(h, sw2d_get_field(h, SW2D_FIELD_VV, vv.data()), "sw2d_get_field");
            write_field("x_velocity", vv, 1.0);  // x = column direction (cu:1436)
        }
        if (su.out_vy == 1) {
            check(h, sw2d_get_field(h, SW2D_FIELD_UU, uu.data()), "sw2d_get_field");
            write_field("y_velocity", uu, -1.0);  // y = north, the negated row direction (cu:1452)
        }
        if (su.out_z == 1) write_field("Elevations", dem.v, 1.0);
        std::fclose(vtk);
        if (su.out_outlet == 1) {  // probe values in cell order (cu:1386-1410)
            int npout = 0;
            const int n_out = (int)probe_km.size();
            for (size_t km = 0; km < ncell; km++)
                for (long pk : probe_km)
                    if ((long)km == pk) {
                        npout++;
                        const double v = first ? ic[km] : hh[km];
                        std::fprintf(wl, npout == n_out ? " %lf\n" : " %lf", v);
                    }
        }
        if (hyd) {
            sw2d_budget b;
            check(h, sw2d_get_budget(h, &b), "sw2d_get_budget");
            const double rate = b.t > hyd_t ? (b.outflow - hyd_v) / (b.t - hyd_t) : 0.0;
            std::fprintf(hyd, "%lf %.9e %.9e\n", b.t, b.outflow, rate);
            hyd_t = b.t;
            hyd_v = b.outflow;
        }
        outputs++;
        first = false;
        if (o.max_outputs >= 0 && outputs >= o.max_outputs) break;
    }
    const double duration = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    std::printf("printf: %g\n", duration);
    FILE *ts = std::fopen((out + "TimeSimu_" + tempo + ".txt").c_str(), "w");
    if (ts) {
        std::fprintf(ts, " %lf\n", duration);
        std::fclose(ts);
    }
    std::fclose(wl);
    if (hyd) std::fclose(hyd);
    sw2d_destroy(h);
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    Opts o;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        auto next = [&]() -> std::string { return i + 1 < argc ? argv[++i] : ""; };
        if (a == "--db") o.db = next();
        else if (a == "--precision") o.precision = next() == "f32" ? SW2D_PREC_F32 : SW2D_PREC_F64;
        else if (a == "--cfl") o.cfl = std::atof(next().c_str());
        else if (a == "--max-outputs") o.max_outputs = std::atol(next().c_str());
        else if (a == "--south-open") o.south_open = true;
        else {
            std::fprintf(stderr, "usage: %s [--db DIR] [--precision f64|f32] [--cfl C] [--south-open] [--max-outputs N]\n",
                         argv[0]);
            return 2;
        }
    }
    std::vector<std::string> t = tokens(o.db + "/dir.txt");  // "dir_number: N" then N names (cu:773-776)
    if (t.size() < 2) {
        std::printf("unknown file - dir.txt\n");
        return 1;
    }
    const int n = std::atoi(t[1].c_str());
    int rc = 0;
    for (int k = 0; k < n && 2 + k < (int)t.size(); k++) rc |= run_case(o, t[2 + k]);
    return rc;
}
