// output.cu -- snapshot output off the time-stepping path.
//
// covof_vtk_write_async writes the files of the reference's vtk_write_step
// (src/module_vtk_writer.f90:90-386, one rank: <dir>/<case>_p0_<step>.vtr and
// <dir>/<case>_<step>.pvtr) from the resident fields without holding up the
// steps that follow:
//   1. on the handle's stream, a device-to-device copy of the fields the files
//      show into a staging area (tens of microseconds even at 4096^2);
//   2. on a side stream, after (1), the copy of the staging area into pinned
//      host memory;
//   3. a host thread waits for (2), formats the ASCII files in the reference's
//      layout (every value as Fortran ES16.8, i.e. "%16.8E") and writes them.
// The next snapshot first joins the previous writer thread, which waited for
// its host copy, so the staging area is reused only after that copy finished;
// the steps that follow a snapshot never wait for its host copy or its file.
//
// covof_history_write_async appends the line of the reference's
// vtk_write_diagnostics (src/module_vtk_writer.f90:392-470) to
// <dir>/<case>_history.csv through the same snapshot; its sums run on the
// host thread in the reference's serial order (host code is built without
// floating-point contraction), so the line matches the reference's digits.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <string>
#include <thread>
#include <vector>

#include "handle.cuh"

using namespace covof;
using namespace covof::host;

namespace {

// fields in the staging area, in this order
enum { S_C, S_CS, S_P, S_RHO, S_MU, S_U, S_V, S_CURV, S_N };

struct Writer {
  std::thread th;
  int status = COVOF_OK;
  double* dstage = nullptr;   // S_N * g doubles on the device
  double* hstage = nullptr;   // S_N * g doubles, pinned
  cudaStream_t io = nullptr;
  cudaEvent_t snap = nullptr, copied = nullptr;
};

void append_es(std::string& out, double x) {
  char buf[40];
  std::snprintf(buf, sizeof(buf), "%16.8E ", x);
  out += buf;
}

// The reference's .vtr and .pvtr files for one rank, from host copies of the
// fields ((nx+2)*(ny+2) each, reference layout).
int write_files(const covof_params& P, const double* const f[S_N], const std::string& dir, const std::string& name,
                int step) {
  const int nx = P.nx, ny = P.ny, W = nx + 2;
  auto at = [&](int q, int i, int j) { return f[q][(size_t)j * W + i]; };
  char step_str[16];
  std::snprintf(step_str, sizeof(step_str), "%06d", step);
  std::string out;
  out.reserve((size_t)nx * ny * 17 * 10 + 4096);
  char line[512];
  out += "<?xml version=\"1.0\"?>\n";
  out += "<VTKFile type=\"RectilinearGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  std::snprintf(line, sizeof(line), "  <RectilinearGrid WholeExtent=\"%d %d %d %d 0 0\">\n", 0, nx, 0, ny);
  out += line;
  std::snprintf(line, sizeof(line), "    <Piece Extent=\"%d %d %d %d 0 0\">\n", 0, nx, 0, ny);
  out += line;
  out += "      <CellData Scalars=\"PhaseIndicator,Pressure,Density,Viscosity,Divergence\" Vectors=\"Velocity\">\n";
  auto scalar = [&](const char* label, auto value) {
    out += "        <DataArray type=\"Float64\" Name=\"";
    out += label;
    out += "\" format=\"ascii\">\n";
    for (int j = 1; j <= ny; ++j) {
      for (int i = 1; i <= nx; ++i) append_es(out, value(i, j));
      out += "\n";
    }
    out += "        </DataArray>\n";
  };
  scalar("PhaseIndicator", [&](int i, int j) { return at(S_C, i, j); });
  scalar("PhaseIndicator_Smoothed", [&](int i, int j) { return at(S_CS, i, j); });
  scalar("Pressure", [&](int i, int j) { return at(S_P, i, j); });
  scalar("Density", [&](int i, int j) { return at(S_RHO, i, j); });
  scalar("Viscosity", [&](int i, int j) { return at(S_MU, i, j); });
  scalar("Divergence", [&](int i, int j) {
    return (at(S_U, i + 1, j) - at(S_U, i, j)) / P.dx + (at(S_V, i, j + 1) - at(S_V, i, j)) / P.dy;
  });
  // no energy equation on this path: the reference's reset value (300 K)
  scalar("Temperature", [&](int, int) { return 300.0; });
  scalar("Curvature", [&](int i, int j) { return at(S_CURV, i, j); });
  out += "        <DataArray type=\"Float64\" Name=\"Velocity\" NumberOfComponents=\"3\" format=\"ascii\">\n";
  for (int j = 1; j <= ny; ++j) {
    for (int i = 1; i <= nx; ++i) {
      append_es(out, 0.5 * (at(S_U, i, j) + at(S_U, i + 1, j)));
      append_es(out, 0.5 * (at(S_V, i, j) + at(S_V, i, j + 1)));
      out += "0.0 ";
    }
    out += "\n";
  }
  out += "        </DataArray>\n";
  out += "      </CellData>\n";
  out += "      <Coordinates>\n";
  out += "        <DataArray type=\"Float64\" Name=\"XCoordinates\" format=\"ascii\">\n";
  for (int i = 0; i <= nx; ++i) append_es(out, (double)i * P.dx);
  out += "\n";
  out += "        </DataArray>\n";
  out += "        <DataArray type=\"Float64\" Name=\"YCoordinates\" format=\"ascii\">\n";
  for (int j = 0; j <= ny; ++j) append_es(out, (double)j * P.dy);
  out += "\n";
  out += "        </DataArray>\n";
  out += "        <DataArray type=\"Float64\" Name=\"ZCoordinates\" format=\"ascii\">\n";
  out += "          0.0\n";
  out += "        </DataArray>\n";
  out += "      </Coordinates>\n";
  out += "    </Piece>\n";
  out += "  </RectilinearGrid>\n";
  out += "</VTKFile>\n";
  const std::string vtr = dir + "/" + name + "_p0_" + step_str + ".vtr";
  FILE* fp = std::fopen(vtr.c_str(), "wb");
  if (!fp) return COVOF_INVALID;
  const bool ok = std::fwrite(out.data(), 1, out.size(), fp) == out.size();
  std::fclose(fp);
  if (!ok) return COVOF_INVALID;

  std::string pv;
  pv += "<?xml version=\"1.0\"?>\n";
  pv += "<VTKFile type=\"PRectilinearGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
  std::snprintf(line, sizeof(line), "  <PRectilinearGrid WholeExtent=\"0 %d 0 %d 0 0\" GhostLevel=\"0\">\n", nx, ny);
  pv += line;
  pv += "    <PCellData Scalars=\"PhaseIndicator,Pressure,Density,Viscosity,Divergence\" Vectors=\"Velocity\">\n";
  for (const char* n : {"PhaseIndicator", "PhaseIndicator_Smoothed", "Pressure", "Density", "Viscosity", "Divergence",
                        "Temperature", "Curvature"}) {
    pv += "      <PDataArray type=\"Float64\" Name=\"";
    pv += n;
    pv += "\"/>\n";
  }
  pv += "      <PDataArray type=\"Float64\" Name=\"Velocity\" NumberOfComponents=\"3\"/>\n";
  pv += "    </PCellData>\n";
  pv += "    <PCoordinates>\n";
  pv += "      <PDataArray type=\"Float64\" Name=\"XCoordinates\"/>\n";
  pv += "      <PDataArray type=\"Float64\" Name=\"YCoordinates\"/>\n";
  pv += "      <PDataArray type=\"Float64\" Name=\"ZCoordinates\"/>\n";
  pv += "    </PCoordinates>\n";
  std::snprintf(line, sizeof(line), "    <Piece Extent=\"%d %d %d %d 0 0\" Source=\"%s_p0_%s.vtr\"/>\n", 0, nx, 0, ny,
                name.c_str(), step_str);
  pv += line;
  pv += "  </PRectilinearGrid>\n";
  pv += "</VTKFile>\n";
  const std::string pvtr = dir + "/" + name + "_" + step_str + ".pvtr";
  fp = std::fopen(pvtr.c_str(), "wb");
  if (!fp) return COVOF_INVALID;
  const bool ok2 = std::fwrite(pv.data(), 1, pv.size(), fp) == pv.size();
  std::fclose(fp);
  return ok2 ? COVOF_OK : COVOF_INVALID;
}

// src/module_vtk_writer.f90:392-470 for one rank: the serial sums in the
// reference's order and the CSV record (I0, then ES14.6 values).
int append_history(const covof_params& P, const double* const f[S_N], const std::string& path, int step,
                   double time, double dt) {
  const int nx = P.nx, ny = P.ny, W = nx + 2;
  auto at = [&](int q, int i, int j) { return f[q][(size_t)j * W + i]; };
  const double dvol = P.dx * P.dy;
  const double T = 300.0;  // no energy equation on this path: the reset temperature
  double vol = 0.0, gvol = 0.0, yint = 0.0, vint = 0.0, mgas = 0.0, pgas = 0.0, ke = 0.0;
  double umax = 0.0, dmax = 0.0;
  for (int j = 1; j <= ny; ++j) {
    const double y_pos = ((double)(j - 1) + 0.5) * P.dy;
    for (int i = 1; i <= nx; ++i) {
      const double c = at(S_C, i, j), pr = at(S_P, i, j);
      const double ib = 1.0 - c;
      vol = vol + ib * dvol;
      yint = yint + y_pos * ib * dvol;
      const double ig = 1.0 - c;
      const double rg = pr / (287.05 * (T > 1.0 ? T : 1.0));
      mgas = mgas + ig * rg * dvol;
      pgas = pgas + ig * pr * dvol;
      gvol = gvol + ig * dvol;
      const double uw = at(S_U, i, j), ue = at(S_U, i + 1, j);
      const double vs = at(S_V, i, j), vn = at(S_V, i, j + 1);
      const double uc = 0.5 * (uw + ue), vc = 0.5 * (vs + vn);
      vint = vint + vc * ib * dvol;
      const double sp2 = uc * uc + vc * vc;
      const double u2p = 0.5 * (uw * uw + ue * ue), v2p = 0.5 * (vs * vs + vn * vn);
      ke = ke + 0.5 * at(S_RHO, i, j) * (u2p + v2p) * dvol;
      const double sp = std::sqrt(sp2);
      if (sp > umax) umax = sp;
      const double dv = std::fabs((ue - uw) / P.dx + (vn - vs) / P.dy);
      if (dv > dmax) dmax = dv;
    }
  }
  const double yc = vol > 1.0e-12 ? yint / vol : 0.0, vcm = vol > 1.0e-12 ? vint / vol : 0.0;
  const double rho_g = gvol > 1.0e-12 ? mgas / gvol : 0.0, p_g = gvol > 1.0e-12 ? pgas / gvol : 0.0;
  char line[512];
  std::snprintf(line, sizeof(line), "%d,%14.6E,%14.6E,%14.6E,%14.6E,%14.6E,%14.6E,%14.6E,%14.6E,%14.6E,%14.6E\n",
                step, time, dt, yc, vcm, vol, ke, umax, dmax, rho_g, p_g);
  FILE* fp = std::fopen(path.c_str(), "ab");
  if (!fp) return COVOF_INVALID;
  const bool ok = std::fputs(line, fp) >= 0;
  std::fclose(fp);
  return ok ? COVOF_OK : COVOF_INVALID;
}

Writer* writer_of(covof_handle* h) { return static_cast<Writer*>(h->writer); }

}  // namespace

namespace covof {
namespace host {

void writer_destroy(covof_handle* h) {
  Writer* w = writer_of(h);
  if (!w) return;
  if (w->th.joinable()) w->th.join();
  if (w->io) cudaStreamSynchronize(w->io);
  dfree(w->dstage);
  if (w->hstage) cudaFreeHost(w->hstage);
  if (w->snap) cudaEventDestroy(w->snap);
  if (w->copied) cudaEventDestroy(w->copied);
  if (w->io) cudaStreamDestroy(w->io);
  delete w;
  h->writer = nullptr;
}

}  // namespace host
}  // namespace covof

extern "C" {

int covof_vtk_wait(covof_handle* h) {
  if (!h) return COVOF_INVALID;
  Writer* w = writer_of(h);
  if (!w) return COVOF_OK;
  if (w->th.joinable()) w->th.join();
  return w->status;
}

}  // extern "C"

namespace {

// Steps (1) and (2) of a snapshot, then `job` on the writer thread with the
// host copies of the fields.  Returns the previous job's status.
template <class Job>
int snapshot_async(covof_handle* h, Job job) {
  CS(ensure_fields(h));
  if (!h->writer) {
    Writer* w = new (std::nothrow) Writer();
    if (!w) return COVOF_INVALID;
    h->writer = w;
    if (cudaStreamCreateWithFlags(&w->io, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->snap, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&w->copied, cudaEventDisableTiming) != cudaSuccess ||
        dalloc(&w->dstage, (size_t)S_N * h->g) != COVOF_OK ||
        cudaMallocHost(&w->hstage, sizeof(double) * S_N * h->g) != cudaSuccess) {
      writer_destroy(h);
      return COVOF_CUDA_ERROR;
    }
  }
  Writer* w = writer_of(h);
  // the previous job is done and its staging copies with it
  if (w->th.joinable()) w->th.join();
  const int prev = w->status;
  w->status = COVOF_OK;
  const size_t bytes = h->g * sizeof(double);
  // (1) snapshot on the handle's stream (after every step enqueued so far)
  const double* src[S_N] = {h->f_C, h->f_Cs, h->f_p, h->f_rho, h->f_mu, h->f_u, h->f_v, h->f_curv};
  for (int q = 0; q < S_N; ++q)
    CK(cudaMemcpyAsync(w->dstage + (size_t)q * h->g, src[q], bytes, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaEventRecord(w->snap, h->stream));
  // (2) host copy on the side stream
  CK(cudaStreamWaitEvent(w->io, w->snap, 0));
  CK(cudaMemcpyAsync(w->hstage, w->dstage, bytes * S_N, cudaMemcpyDeviceToHost, w->io));
  CK(cudaEventRecord(w->copied, w->io));
  // (the next snapshot joins this job, which waited for the host copy, before
  // its device copies reuse the staging area)
  // (3) the job on a host thread
  double* hs = w->hstage;
  const size_t g = h->g;
  cudaEvent_t copied = w->copied;
  w->th = std::thread([w, hs, g, copied, job]() {
    if (cudaEventSynchronize(copied) != cudaSuccess) { w->status = COVOF_CUDA_ERROR; return; }
    const double* f[S_N];
    for (int q = 0; q < S_N; ++q) f[q] = hs + (size_t)q * g;
    w->status = job(f);
  });
  return prev;
}

}  // namespace

extern "C" {

int covof_vtk_write_async(covof_handle* h, const char* dir, const char* case_name, int step) {
  if (!h || !dir || !case_name || step < 0) return COVOF_INVALID;
  const covof_params P = h->prm;
  const std::string d(dir), n(case_name);
  return snapshot_async(h, [P, d, n, step](const double* const* f) {
    std::error_code ec;
    std::filesystem::create_directories(d, ec);  // vtk_init's mkdir -p
    return write_files(P, f, d, n, step);
  });
}

// vtk_init's history file (src/module_vtk_writer.f90:61-70): the directory,
// then <dir>/<case>_history.csv replaced by its header line.
int covof_history_open(covof_handle* h, const char* dir, const char* case_name) {
  if (!h || !dir || !case_name) return COVOF_INVALID;
  CS(covof_vtk_wait(h));
  std::error_code ec;
  std::filesystem::create_directories(dir, ec);
  const std::string path = std::string(dir) + "/" + case_name + "_history.csv";
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) return COVOF_INVALID;
  std::fputs("step,time,dt,center_of_mass_y,rise_velocity,bubble_volume,kinetic_energy,max_u,max_div,"
             "avg_rho_gas,avg_p_gas\n", fp);
  std::fclose(fp);
  return COVOF_OK;
}

int covof_history_write_async(covof_handle* h, const char* dir, const char* case_name, int step, double time,
                              double dt) {
  if (!h || !dir || !case_name) return COVOF_INVALID;
  const covof_params P = h->prm;
  const std::string path = std::string(dir) + "/" + case_name + "_history.csv";
  return snapshot_async(h, [P, path, step, time, dt](const double* const* f) {
    return append_history(P, f, path, step, time, dt);
  });
}

}  // extern "C"

COVOF_UNIT_HOOKS(output)
