// Runs a JSON deck of the reference's explicit driver on the GPU: the
// counterpart of `weldform_exp deck.json` (src/explicit/main.C:125-1005 then
// Domain_d::SolveChungHulbert). Writes <deck>_NNNNN.vtk at t = 0 and every
// outTime (from snapshots, written while the next steps run), <deck>_res.json
// listing them (ResultsJson, Solver_explicit.C:48-78)
// and, with --energy, <deck>_energy.csv with t, Eint, Ekin per step; prints a
// one-line JSON summary.
//
// usage: wf_deck_solve deck.json [--mixed] [--no-vtk] [--energy]
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "wf.h"

namespace {

int fail(wf_domain *d, wf_status s, const char *what) {
  std::fprintf(stderr, "%s: %s (%s)\n", what, wf_status_string(s), d ? wf_last_error(d) : "");
  if (d) wf_domain_destroy(d);
  return 1;
}

std::string vtk_name(const std::string &base, int idx) {
  char buf[16];
  std::snprintf(buf, sizeof(buf), "_%05d.vtk", idx);
  return base + buf;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s deck.json [--mixed] [--no-vtk] [--energy]\n", argv[0]);
    return 2;
  }
  const std::string path = argv[1];
  bool mixed = false, vtk = true, energy = false;
  for (int i = 2; i < argc; i++) {
    if (!std::strcmp(argv[i], "--mixed")) mixed = true;
    else if (!std::strcmp(argv[i], "--no-vtk")) vtk = false;
    else if (!std::strcmp(argv[i], "--energy")) energy = true;
  }
  const std::string base = path.substr(0, path.find_last_of('.'));
  wf_domain *d = nullptr;
  wf_status s = wf_domain_create(&d);
  if (s) return fail(nullptr, s, "wf_domain_create");
  if (mixed && (s = wf_set_precision(d, WF_MIXED))) return fail(d, s, "wf_set_precision");
  wf_deck_info info;
  char err[512] = {0};
  if ((s = wf_load_deck(d, path.c_str(), &info, err, sizeof(err)))) {
    std::fprintf(stderr, "%s: %s\n", path.c_str(), err);
    wf_domain_destroy(d);
    return 1;
  }
  if (energy && (s = wf_set_energy_history(d, 1))) return fail(d, s, "wf_set_energy_history");
  const auto t0 = std::chrono::steady_clock::now();
  if ((s = wf_init(d))) return fail(d, s, "wf_init");
  std::vector<std::pair<std::string, double>> files;
  // outputs go through snapshots: the state of an output time is copied to
  // host memory beside the next steps, and its file is written while the GPU
  // runs them (the reference loop stops for each output instead)
  int32_t pending = -1;
  double pending_t = 0.0;
  auto flush = [&]() -> wf_status {
    if (pending < 0) return WF_OK;
    const std::string f = vtk_name(base, (int)files.size());
    const wf_status ws = wf_write_snapshot_vtk(d, pending, f.c_str());
    pending = -1;
    if (ws) return ws;
    files.emplace_back(f, pending_t);
    FILE *j = std::fopen((base + "_res.json").c_str(), "w");
    if (j) {
      std::fprintf(j, "{\n  \"vtk_files\": [\n");
      for (size_t i = 0; i < files.size(); i++)
        std::fprintf(j, "    { \"file\": \"%s\", \"time\": %.9g }%s\n", files[i].first.c_str(),
                     files[i].second, i + 1 < files.size() ? "," : "");
      std::fprintf(j, "  ]\n}\n");
      std::fclose(j);
    }
    return WF_OK;
  };
  auto write = [&](double t) -> wf_status {
    if (!vtk) return WF_OK;
    int32_t slot = -1;
    wf_status ws = wf_snapshot(d, &slot);   // queued after the steps run so far
    if (ws) return ws;
    ws = flush();                           // the previous output, written meanwhile
    pending = slot;
    pending_t = t;
    return ws;
  };
  if ((s = write(0.0))) return fail(d, s, "wf_snapshot");
  // the loop runs while Time < end time; outputs when Time reaches tout
  double t = 0.0, tout = info.out_time > 0.0 ? info.out_time : info.end_time;
  int64_t steps = 0;
  while (t < info.end_time) {
    int64_t n = 0;
    double tt = t;
    while (tt < info.end_time && (tt < tout || n == 0)) {
      tt += info.dt;
      n++;
    }
    if ((s = wf_run(d, n))) return fail(d, s, "wf_run");
    steps += n;
    int64_t st = 0;
    wf_get_time(d, &t, &st);
    if (t >= tout || t >= info.end_time) {
      if ((s = write(t))) return fail(d, s, "wf_snapshot");
      while (tout <= t) tout += info.out_time > 0.0 ? info.out_time : info.end_time;
    }
  }
  if ((s = flush())) return fail(d, s, "wf_write_snapshot_vtk");
  if ((s = wf_sync(d))) return fail(d, s, "wf_sync");
  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (energy) {
    std::vector<double> ek(steps), ei(steps);
    int64_t n = 0;
    if ((s = wf_get_energy_history(d, ek.data(), ei.data(), steps, &n)))
      return fail(d, s, "wf_get_energy_history");
    FILE *f = std::fopen((base + "_energy.csv").c_str(), "w");
    if (f) {
      std::fprintf(f, "t,Eint,Ekin\n");
      for (int64_t i = 0; i < n && i < steps; i++)
        std::fprintf(f, "%.9g,%.9g,%.9g\n", (i + 1) * info.dt, ei[i], ek[i]);
      std::fclose(f);
    }
  }
  std::printf("{\"deck\": \"%s\", \"steps\": %lld, \"time\": %.9g, \"dt\": %.9g, \"elements\": %lld, "
              "\"nodes\": %lld, \"vtk_files\": %zu, \"seconds\": %.3f}\n",
              path.c_str(), (long long)steps, t, info.dt, (long long)info.ne, (long long)info.nn,
              files.size(), secs);
  wf_domain_destroy(d);
  return 0;
}
