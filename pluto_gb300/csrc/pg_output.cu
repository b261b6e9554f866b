// Output files written from the device: the .dbl / .flt / .vtk branches of
// PLUTO's WriteData (Src/write_data.c:29-330) and its ".out" record
// (Src/write_data.c:360-385), plus the data part of RestartFromFile
// (Src/restart.c:17-150).
//
// Byte layout, as a serial reference run writes it:
//   FileWriteData (Src/bin_io.c:216-259): per variable the interior
//     [k][j][i], a staggered component one longer along its own axis (faces
//     BEG-1 .. END, i.e. from the left face of the first zone);
//   .dbl: native doubles; .flt: Convert_dbl2flt (Src/bin_io.c:51-83),
//     (float)(v*unit), native byte order;
//   .vtk: WriteVTK_Header (Src/write_vtk.c) text + big-endian float node
//     coordinates of a rectilinear grid, then VECTORS (Float_Vect triples
//     (float)v*unit over the first DIMENSIONS components, zero beyond) and
//     SCALARS blocks in big-endian floats;
//   single_file: data.NNNN.<ext>; multiple_files: <var>.NNNN.<ext>, VTK
//     vectors in vfield / bfield.NNNN.vtk.
//
// Pipeline: the dumped variables are packed in file order into a device
// staging buffer by one kernel per variable on the solver's stream; a copy
// stream waits on an event after them and moves the buffer to pinned host
// memory; a writer thread waits on the copy's event and writes the files and
// the record.  Two staging slots; a third output waits for the oldest.
#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pg_internal.h"
#include "pg_dw.cuh"

float* mixed_cell_array(pg::Solver* S, int nv);
float* mixed_face_array(pg::Solver* S, int d);

namespace pg {

enum : int { K_F64 = 0, K_F32 = 1, K_F32BE = 2, K_VEC3BE = 3 };

struct PackSeg {
  const void* src[3];  // cell or face arrays of the solver (T elements)
  int ncomp;           // components read (vectors: DIMENSIONS)
  int kind;
  double unit;
  unsigned char* dst;
  int lo[3], n[3];     // box in the solver's index space
};

__device__ __forceinline__ unsigned bswap32(unsigned x) { return __byte_perm(x, 0u, 0x0123); }

// float <-> double in integer arithmetic (pg_dw.cuh: exact widening,
// round-to-nearest-even narrowing, checked against the IEEE conversions by
// pg_selftest_conversions): the hardware conversions issue on the FP64 pipe
__device__ __forceinline__ double to_f64(float v) { return widen(v); }
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ float to_f32(float v, double unit) { return unit == 1.0 ? v : narrow(widen(v) * unit); }
__device__ __forceinline__ float to_f32(double v, double unit) { return narrow(unit == 1.0 ? v : v * unit); }

// one output variable of the interior box into the staging buffer: threads
// along i, blockIdx.y over j, blockIdx.z striding over k, four k planes per
// pass with every load issued before the stores (no integer division
// anywhere: it issues on the FP64 pipe on this GPU)
constexpr int kPackPlanes = 4;
template <class T>
__global__ void k_pack(PackSeg s, Geom g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.n[0]) return;
  const int nc = s.kind == K_VEC3BE ? s.ncomp : 1;
  for (int j = blockIdx.y; j < s.n[1]; j += gridDim.y)
    for (int k0 = blockIdx.z; k0 < s.n[2]; k0 += kPackPlanes * gridDim.z) {
      T v[kPackPlanes][3];
#pragma unroll
      for (int u = 0; u < kPackPlanes; u++) {
        const int k = k0 + u * gridDim.z;
        const long long c = cidx(g, s.lo[2] + k, s.lo[1] + j, s.lo[0] + i);
#pragma unroll
        for (int m = 0; m < 3; m++)
          if (k < s.n[2] && m < nc) v[u][m] = ((const T*)s.src[m])[c];
      }
#pragma unroll
      for (int u = 0; u < kPackPlanes; u++) {
        const int k = k0 + u * gridDim.z;
        if (k >= s.n[2]) break;
        const long long q = ((long long)k * s.n[1] + j) * s.n[0] + i;
        if (s.kind == K_F64) {
          ((double*)s.dst)[q] = to_f64(v[u][0]);
        } else if (s.kind == K_VEC3BE) {  // (float)v * unit, stored as float (write_vtk.c)
          unsigned* o = (unsigned*)s.dst + 3 * q;
#pragma unroll
          for (int m = 0; m < 3; m++) {
            const float f = m < nc ? to_f32(to_f32(v[u][m], 1.0), s.unit) : 0.0f;
            o[m] = bswap32(__float_as_uint(f));
          }
        } else {
          const unsigned b = __float_as_uint(to_f32(v[u][0], s.unit));
          ((unsigned*)s.dst)[q] = s.kind == K_F32BE ? bswap32(b) : b;
        }
      }
    }
}

// a file: literal byte pieces and spans of the packed buffer, in order
struct Piece {
  std::string bytes;
  size_t off = 0, len = 0;
  bool span = false;
};
struct FilePlan {
  std::string path;
  std::vector<Piece> pieces;
};
struct Plan {
  std::vector<FilePlan> files;
  std::vector<PackSeg> segs;  // dst holds the byte offset until a slot is bound
  size_t bytes = 0;
  std::string out_path, record;
  int nfile = 0;
  bool write_record = false;
};
struct Slot {
  unsigned char* dev = nullptr;
  unsigned char* host = nullptr;
  size_t cap = 0;
  bool busy = false;
};
struct Job {
  Plan plan;
  int slot = 0;
  cudaEvent_t copied = nullptr;
};
struct OutputState {
  cudaStream_t copy = nullptr;
  int device = 0;
  Slot slots[2];
  Slot dl;                           // staging of pg_download_async
  cudaEvent_t dl_packed = nullptr, dl_done = nullptr;
  bool dl_pending = false;
  std::thread worker;
  std::mutex m;
  std::condition_variable cv;
  std::deque<Job> q;
  int pending = 0;
  bool stop = false;
  int error = PG_OK;
  std::string error_msg;
};

static const char* ext_of(int format) { return format == PG_OUT_DBL ? "dbl" : (format == PG_OUT_FLT ? "flt" : "vtk"); }

static void be32(std::string& s, float f) {
  unsigned u;
  memcpy(&u, &f, 4);
  const char b[4] = {(char)(u >> 24), (char)(u >> 16), (char)(u >> 8), (char)u};
  s.append(b, 4);
}

// WriteVTK_Header (Src/write_vtk.c), VTK_RECTILINEAR_GRID, VTK_TIME_INFO NO
static std::string vtk_header(const Geom& g, const pg_output* o) {
  const int dims = g.dims;
  const int nx1 = g.nx[0], nx2 = dims >= 2 ? g.nx[1] : 1, nx3 = dims == 3 ? g.nx[2] : 1;
  const int n[3] = {nx1 + 1, nx2 + (dims >= 2), nx3 + (dims == 3)};
  char line[256];
  std::string h = "# vtk DataFile Version 2.0\nPLUTO 4.3 VTK Data\nBINARY\nDATASET RECTILINEAR_GRID\n";
  snprintf(line, sizeof line, "DIMENSIONS %d %d %d\n", n[0], n[1], n[2]);
  h += line;
  static const char* axis[3] = {"X", "Y", "Z"};
  for (int d = 0; d < 3; d++) {
    snprintf(line, sizeof line, "%s%s_COORDINATES %d float\n", d ? "\n" : "", axis[d], n[d]);
    h += line;
    for (int m = 0; m < n[d]; m++) be32(h, (d == 2 && dims == 2) ? 0.0f : (float)o->xnode[d][m]);
  }
  snprintf(line, sizeof line, "\nCELL_DATA %d\n", nx1 * nx2 * nx3);
  h += line;
  return h;
}

static int build_plan(const Solver* S, const pg_output* o, Plan& P, std::string& err) {
  const Geom& g = S->g;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  if (o->format < PG_OUT_DBL || o->format > PG_OUT_VTK) return err = "unknown output format", PG_ERR_INVALID;
  if (o->nvar < 0 || o->nvar > PG_OUT_MAX_VARS) return err = "nvar out of range", PG_ERR_INVALID;
  if (!o->dir) return err = "null output directory", PG_ERR_INVALID;
  if ((long long)(g.nx[0] + 1) * (g.nx[1] + 1) * (g.nx[2] + 1) >= (1LL << 31))
    return err = "a variable of more than 2^31 elements", PG_ERR_TOO_LARGE;
  const char* ext = ext_of(o->format);
  std::string header;
  if (o->format == PG_OUT_VTK) {
    for (int d = 0; d < 3; d++)
      if (!o->xnode[d]) return err = "VTK output needs the node coordinates xnode[0..2]", PG_ERR_INVALID;
    header = vtk_header(g, o);
  }
  char path[1024];
  auto add_seg = [&](int id, int kind, int ncomp, double unit) -> Piece {
    PackSeg s;
    memset(&s, 0, sizeof s);
    const int fd = id >= 8 ? id - 8 : -1;
    for (int ax = 0; ax < 3; ax++) {
      const bool stag = ax == fd && ax < g.dims;
      s.lo[ax] = g.beg[ax] - (stag ? 1 : 0);
      s.n[ax] = g.nx[ax] + (stag ? 1 : 0);
    }
    s.kind = kind;
    s.ncomp = ncomp;
    s.unit = unit;
    for (int m = 0; m < 3; m++) s.src[m] = (const void*)(intptr_t)(m < ncomp ? id + m : -1);  // bound later
    const size_t esz = kind == K_F64 ? 8 : (kind == K_VEC3BE ? 12 : 4);
    const size_t len = (size_t)s.n[0] * s.n[1] * s.n[2] * esz;
    P.bytes = (P.bytes + 15) & ~(size_t)15;
    s.dst = (unsigned char*)(uintptr_t)P.bytes;
    P.segs.push_back(s);
    Piece pc;
    pc.span = true;
    pc.off = P.bytes;
    pc.len = len;
    P.bytes += len;
    return pc;
  };
  auto lit = [](const std::string& b) {
    Piece pc;
    pc.bytes = b;
    return pc;
  };
  FilePlan single;
  if (o->single_file) {
    snprintf(path, sizeof path, "%s/data.%04d.%s", o->dir, o->nfile, ext);
    single.path = path;
    if (o->format == PG_OUT_VTK) single.pieces.push_back(lit(header));
  }
  // VTK writes every vector, then every scalar (Src/write_data.c:246-262)
  const int passes = o->format == PG_OUT_VTK ? 2 : 1;
  for (int pass = 0; pass < passes; pass++)
    for (int nv = 0; nv < o->nvar; nv++) {
      const int dump = o->dump[nv], id = o->var[nv];
      if (!dump) continue;
      if (id < 0 || id > 10) return err = "output var id out of range", PG_ERR_INVALID;
      const int fd = id >= 8 ? id - 8 : -1;
      if (fd >= 0 && (!ct || fd >= g.dims)) return err = "no staggered component for this output var", PG_ERR_INVALID;
      if (fd >= 0 && o->format != PG_OUT_DBL)
        return err = "staggered fields are written in .dbl files only", PG_ERR_INVALID;
      const char* name = o->name[nv] ? o->name[nv] : "";
      const double unit = o->format == PG_OUT_DBL ? 1.0 : o->unit[nv];
      if (o->format == PG_OUT_VTK) {
        const bool vec = dump == PG_OUT_VECTOR;
        if (vec != (pass == 0)) continue;
        if (!vec && dump != 1) continue;  // WriteData writes scalars with dump_var == YES only
        FilePlan mf;
        Piece body;
        std::string head;
        char h[512];
        if (vec) {
          const bool vel = !strcmp(name, "vx1"), mag = !strcmp(name, "bx1");
          if (!o->single_file && !vel && !mag) return err = "unknown vector type in VTK output", PG_ERR_INVALID;
          if (!vel && !mag) continue;  // WriteVTK_Vector writes nothing for it
          if (id + g.dims - 1 > 7) return err = "VTK vector components out of range", PG_ERR_INVALID;
          snprintf(h, sizeof h, "\nVECTORS %dD_%s_Field float\n", g.dims, vel ? "Velocity" : "Magnetic");
          head = h;
          body = add_seg(id, K_VEC3BE, g.dims, o->unit[nv]);
          snprintf(path, sizeof path, "%s/%s.%04d.%s", o->dir, vel ? "vfield" : "bfield", o->nfile, ext);
        } else {
          snprintf(h, sizeof h, "\nSCALARS %s float\nLOOKUP_TABLE default\n", name);
          head = h;
          body = add_seg(id, K_F32BE, 1, unit);
          snprintf(path, sizeof path, "%s/%s.%04d.%s", o->dir, name, o->nfile, ext);
        }
        FilePlan& f = o->single_file ? single : mf;
        if (!o->single_file) {
          mf.path = path;
          mf.pieces.push_back(lit(header));
        }
        f.pieces.push_back(lit(head));
        f.pieces.push_back(body);
        if (!o->single_file) P.files.push_back(mf);
      } else {
        const Piece body = add_seg(id, o->format == PG_OUT_DBL ? K_F64 : K_F32, 1, unit);
        if (o->single_file) {
          single.pieces.push_back(body);
        } else {
          FilePlan mf;
          snprintf(path, sizeof path, "%s/%s.%04d.%s", o->dir, name, o->nfile, ext);
          mf.path = path;
          mf.pieces.push_back(body);
          P.files.push_back(mf);
        }
      }
    }
  if (o->single_file) P.files.insert(P.files.begin(), single);
  // the ".out" record (Src/write_data.c:360-385)
  P.write_record = o->write_record != 0;
  P.nfile = o->nfile;
  snprintf(path, sizeof path, "%s/%s.out", o->dir, ext);
  P.out_path = path;
  char rec[512];
  snprintf(rec, sizeof rec, "%d %12.6e %12.6e %ld ", o->nfile, o->time, o->dt, o->step);
  P.record = rec;
  P.record += o->single_file ? "single_file " : "multiple_files ";
  const unsigned one = 1;
  P.record += *(const unsigned char*)&one ? "little " : "big ";
  for (int nv = 0; nv < o->nvar; nv++)
    if (o->dump[nv]) {
      P.record += o->name[nv] ? o->name[nv] : "";
      P.record += " ";
    }
  P.record += "\n";
  return PG_OK;
}

static int write_record(const Plan& P) {
  FILE* f;
  if (P.nfile == 0) {
    f = fopen(P.out_path.c_str(), "w");
  } else {
    f = fopen(P.out_path.c_str(), "r+");
    if (!f) f = fopen(P.out_path.c_str(), "w");
    char line[512];
    for (int n = 0; f && n < P.nfile; n++)
      if (!fgets(line, sizeof line, f)) break;
    if (f) fseek(f, ftell(f), SEEK_SET);
  }
  if (!f) return -1;
  const bool ok = fwrite(P.record.data(), 1, P.record.size(), f) == P.record.size();
  return (fclose(f) == 0 && ok) ? 0 : -1;
}

static void worker_main(OutputState* O) {
  cudaSetDevice(O->device);
  for (;;) {
    Job job;
    {
      std::unique_lock<std::mutex> lk(O->m);
      O->cv.wait(lk, [&] { return O->stop || !O->q.empty(); });
      if (O->q.empty()) return;
      job = std::move(O->q.front());
      O->q.pop_front();
    }
    std::string err;
    if (cudaEventSynchronize(job.copied) != cudaSuccess) err = "device-to-host copy of an output failed";
    cudaEventDestroy(job.copied);
    const unsigned char* host = O->slots[job.slot].host;
    for (size_t fi = 0; err.empty() && fi < job.plan.files.size(); fi++) {
      const FilePlan& fp = job.plan.files[fi];
      FILE* f = fopen(fp.path.c_str(), "wb");
      if (!f) {
        err = "cannot open " + fp.path;
        break;
      }
      bool ok = true;
      for (const Piece& pc : fp.pieces) {
        if (pc.span) ok = ok && fwrite(host + pc.off, 1, pc.len, f) == pc.len;
        else ok = ok && fwrite(pc.bytes.data(), 1, pc.bytes.size(), f) == pc.bytes.size();
      }
      if (fclose(f) != 0 || !ok) err = "write error on " + fp.path;
    }
    if (err.empty() && job.plan.write_record && write_record(job.plan)) err = "cannot update " + job.plan.out_path;
    {
      std::lock_guard<std::mutex> lk(O->m);
      O->slots[job.slot].busy = false;
      O->pending--;
      if (!err.empty() && O->error == PG_OK) {
        O->error = PG_ERR_INVALID;
        O->error_msg = err;
      }
    }
    O->cv.notify_all();
  }
}

static OutputState* output_state(Solver* S) {
  if (S->out) return (OutputState*)S->out;
  OutputState* O = new OutputState();
  cudaGetDevice(&O->device);
  if (cudaStreamCreateWithFlags(&O->copy, cudaStreamNonBlocking) != cudaSuccess) {
    delete O;
    return nullptr;
  }
  O->worker = std::thread(worker_main, O);
  S->out = O;
  return O;
}

static int wait_all(OutputState* O, std::string& msg) {
  std::unique_lock<std::mutex> lk(O->m);
  O->cv.wait(lk, [&] { return O->pending == 0; });
  const int rc = O->error;
  msg = O->error_msg;
  O->error = PG_OK;
  O->error_msg.clear();
  return rc;
}

}  // namespace pg

using namespace pg;

// rows of 128 threads; j over gridDim.y, k strided over gridDim.z so that
// about sixteen blocks per SM are resident
static void launch_pack(const PackSeg& s, const Geom& g, bool is_float, cudaStream_t st) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 1;
  }
  constexpr int kPackThreads = 128;
  const unsigned gx = (unsigned)((s.n[0] + kPackThreads - 1) / kPackThreads);
  const unsigned gy = (unsigned)std::min(s.n[1], 65535);
  const long long per_z = (long long)gx * gy;
  const unsigned gz = (unsigned)std::max<long long>(
      1, std::min<long long>({((long long)s.n[2] + kPackPlanes - 1) / kPackPlanes,
                              (16LL * nsm + per_z - 1) / per_z, 65535LL}));
  const dim3 grid(gx, gy, gz);
  if (is_float) k_pack<float><<<grid, kPackThreads, 0, st>>>(s, g);
  else k_pack<double><<<grid, kPackThreads, 0, st>>>(s, g);
}

void pg::output_free(Solver* S) {
  OutputState* O = (OutputState*)S->out;
  if (!O) return;
  std::string msg;
  wait_all(O, msg);
  {
    std::lock_guard<std::mutex> lk(O->m);
    O->stop = true;
  }
  O->cv.notify_all();
  if (O->worker.joinable()) O->worker.join();
  if (O->dl_pending) cudaEventSynchronize(O->dl_done);
  for (Slot& s : O->slots) {
    if (s.dev) cudaFree(s.dev);
    if (s.host) cudaFreeHost(s.host);
  }
  if (O->dl.dev) cudaFree(O->dl.dev);
  if (O->dl_packed) cudaEventDestroy(O->dl_packed);
  if (O->dl_done) cudaEventDestroy(O->dl_done);
  if (O->copy) cudaStreamDestroy(O->copy);
  delete O;
  S->out = nullptr;
}

static int bind_sources(Solver* S, PackSeg& s, bool& is_float) {
  const bool f64 = S->cfg.precision == PG_FP64;
  is_float = !f64;
  for (int m = 0; m < 3; m++) {
    const intptr_t id = (intptr_t)s.src[m];
    if (id < 0) {
      s.src[m] = nullptr;
      continue;
    }
    if (id >= 8) s.src[m] = f64 ? (const void*)S->Bs[id - 8] : (const void*)mixed_face_array(S, (int)id - 8);
    else s.src[m] = f64 ? (const void*)S->V[id] : (const void*)mixed_cell_array(S, (int)id);
    if (!s.src[m]) return PG_ERR_INVALID;
  }
  return PG_OK;
}

extern "C" int pg_write_output(pg_solver* h, const pg_output* o) {
  if (!h || !o) {
    set_last_error("pg_write_output: null argument");
    return PG_ERR_INVALID;
  }
  Solver* S = &h->S;
  if (S->cfg.precision == PG_FP64_TANGENT || S->cfg.precision == PG_FP64_DD) {
    set_last_error("pg_write_output: FP64 and mixed precisions only");
    return PG_ERR_INVALID;
  }
  Plan P;
  std::string err;
  int rc = build_plan(S, o, P, err);
  if (rc) {
    set_last_error(("pg_write_output: " + err).c_str());
    return rc;
  }
  OutputState* O = output_state(S);
  if (!O) {
    set_last_error("pg_write_output: cannot create the copy stream");
    return PG_ERR_CUDA;
  }
  int slot = -1;
  {
    std::unique_lock<std::mutex> lk(O->m);
    O->cv.wait(lk, [&] { return !O->slots[0].busy || !O->slots[1].busy; });
    slot = !O->slots[0].busy ? 0 : 1;
    O->slots[slot].busy = true;
    O->pending++;
  }
  Slot& sl = O->slots[slot];
  auto release = [&](int code, const char* msg) {
    {
      std::lock_guard<std::mutex> lk(O->m);
      sl.busy = false;
      O->pending--;
    }
    O->cv.notify_all();
    set_last_error(msg);
    return code;
  };
  if (sl.cap < P.bytes) {
    if (sl.dev) cudaFree(sl.dev);
    if (sl.host) cudaFreeHost(sl.host);
    sl.dev = sl.host = nullptr;
    sl.cap = 0;
    if (cudaMalloc(&sl.dev, P.bytes) != cudaSuccess) return release(PG_ERR_NOMEM, "pg_write_output: staging buffer");
    if (cudaHostAlloc(&sl.host, P.bytes, cudaHostAllocDefault) != cudaSuccess) {
      cudaFree(sl.dev);
      sl.dev = nullptr;
      return release(PG_ERR_NOMEM, "pg_write_output: pinned host buffer");
    }
    sl.cap = P.bytes;
  }
  for (PackSeg& s : P.segs) {
    bool is_float = false;
    if (bind_sources(S, s, is_float)) return release(PG_ERR_INVALID, "pg_write_output: state array missing");
    s.dst = sl.dev + (uintptr_t)s.dst;
    launch_pack(s, S->g, is_float, S->stream);
  }
  cudaEvent_t packed = nullptr, copied = nullptr;
  if (cudaGetLastError() != cudaSuccess || cudaEventCreateWithFlags(&packed, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&copied, cudaEventDisableTiming) != cudaSuccess)
    return release(PG_ERR_CUDA, "pg_write_output: pack launch");
  cudaEventRecord(packed, S->stream);
  cudaStreamWaitEvent(O->copy, packed, 0);
  if (P.bytes) cudaMemcpyAsync(sl.host, sl.dev, P.bytes, cudaMemcpyDeviceToHost, O->copy);
  cudaEventRecord(copied, O->copy);
  cudaEventDestroy(packed);
  if (cudaGetLastError() != cudaSuccess) {
    cudaEventDestroy(copied);
    return release(PG_ERR_CUDA, "pg_write_output: device-to-host copy");
  }
  {
    std::lock_guard<std::mutex> lk(O->m);
    Job j;
    j.plan = std::move(P);
    j.slot = slot;
    j.copied = copied;
    O->q.push_back(std::move(j));
  }
  O->cv.notify_all();
  return PG_OK;
}

extern "C" int pg_output_wait(pg_solver* h) {
  if (!h) {
    set_last_error("pg_output_wait: null argument");
    return PG_ERR_INVALID;
  }
  OutputState* O = (OutputState*)h->S.out;
  if (!O) return PG_OK;
  std::string msg;
  const int rc = wait_all(O, msg);
  if (rc) set_last_error(("pg_output_wait: " + msg).c_str());
  return rc;
}

extern "C" int pg_read_output(pg_solver* h, const pg_output* o) {
  if (!h || !o) {
    set_last_error("pg_read_output: null argument");
    return PG_ERR_INVALID;
  }
  Solver* S = &h->S;
  if (o->format != PG_OUT_DBL) {
    set_last_error("pg_read_output: restarts read .dbl files");
    return PG_ERR_INVALID;
  }
  Plan P;
  std::string err;
  int rc = build_plan(S, o, P, err);
  if (rc) {
    set_last_error(("pg_read_output: " + err).c_str());
    return rc;
  }
  if (S->out) {  // an earlier output of these files must be on disk first
    std::string msg;
    if ((rc = wait_all((OutputState*)S->out, msg))) {
      set_last_error(("pg_read_output: " + msg).c_str());
      return rc;
    }
  }
  unsigned char* host = nullptr;
  if (P.bytes && cudaHostAlloc(&host, P.bytes, cudaHostAllocDefault) != cudaSuccess) {
    set_last_error("pg_read_output: pinned host buffer");
    return PG_ERR_NOMEM;
  }
  for (const FilePlan& fp : P.files) {
    FILE* f = fopen(fp.path.c_str(), "rb");
    if (!f) {
      err = "cannot open " + fp.path;
      break;
    }
    for (const Piece& pc : fp.pieces)
      if (pc.span && fread(host + pc.off, 1, pc.len, f) != pc.len) err = "short file " + fp.path;
    fclose(f);
    if (!err.empty()) break;
  }
  if (err.empty()) {
    const double* vars[8] = {};
    const double* faces[3] = {};
    size_t si = 0;
    for (int nv = 0; nv < o->nvar; nv++) {
      if (!o->dump[nv]) continue;
      const double* p = (const double*)(host + (uintptr_t)P.segs[si++].dst);
      if (o->var[nv] >= 8) faces[o->var[nv] - 8] = p;
      else vars[o->var[nv]] = p;
    }
    rc = pg_upload(h, vars, faces, PG_LAYOUT_INTERIOR);
  } else {
    set_last_error(("pg_read_output: " + err).c_str());
    rc = PG_ERR_INVALID;
  }
  if (host) cudaFreeHost(host);
  return rc;
}

// Asynchronous download of the state (interior layout): pack kernels on the
// solver's stream write the FP64 interior of every requested array into a
// device staging buffer, then the copy stream moves each array to the
// caller's host memory while the next steps run.
extern "C" int pg_download_async(pg_solver* h, double* const vars[8], double* const faces[3]) {
  if (!h || !vars) {
    set_last_error("pg_download_async: null argument");
    return PG_ERR_INVALID;
  }
  Solver* S = &h->S;
  if (S->cfg.precision == PG_FP64_TANGENT || S->cfg.precision == PG_FP64_DD) {
    set_last_error("pg_download_async: FP64 and mixed precisions only");
    return PG_ERR_INVALID;
  }
  OutputState* O = output_state(S);
  if (!O) {
    set_last_error("pg_download_async: cannot create the copy stream");
    return PG_ERR_CUDA;
  }
  const Geom& g = S->g;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  if ((long long)(g.nx[0] + 1) * (g.nx[1] + 1) * (g.nx[2] + 1) >= (1LL << 31)) {
    set_last_error("pg_download_async: a variable of more than 2^31 elements");
    return PG_ERR_TOO_LARGE;
  }
  std::vector<PackSeg> segs;
  std::vector<double*> dst;
  size_t bytes = 0;
  for (int id = 0; id < 11; id++) {
    double* host = id < 8 ? vars[id] : (faces && ct && id - 8 < g.dims ? faces[id - 8] : nullptr);
    if (!host) continue;
    PackSeg s;
    memset(&s, 0, sizeof s);
    const int fd = id >= 8 ? id - 8 : -1;
    for (int ax = 0; ax < 3; ax++) {
      const bool stag = ax == fd && ax < g.dims;
      s.lo[ax] = g.beg[ax] - (stag ? 1 : 0);
      s.n[ax] = g.nx[ax] + (stag ? 1 : 0);
    }
    s.kind = K_F64;
    s.ncomp = 1;
    s.unit = 1.0;
    s.src[0] = (const void*)(intptr_t)id;
    s.src[1] = s.src[2] = (const void*)(intptr_t)-1;
    bytes = (bytes + 15) & ~(size_t)15;
    s.dst = (unsigned char*)(uintptr_t)bytes;
    bytes += (size_t)s.n[0] * s.n[1] * s.n[2] * sizeof(double);
    segs.push_back(s);
    dst.push_back(host);
  }
  if (O->dl_pending) {  // the staging buffer is still being copied out
    if (cudaEventSynchronize(O->dl_done) != cudaSuccess) {
      set_last_error("pg_download_async: previous copy failed");
      return PG_ERR_CUDA;
    }
    O->dl_pending = false;
  }
  if (O->dl.cap < bytes) {
    if (O->dl.dev) cudaFree(O->dl.dev);
    O->dl.dev = nullptr;
    O->dl.cap = 0;
    if (cudaMalloc(&O->dl.dev, bytes) != cudaSuccess) {
      set_last_error("pg_download_async: staging buffer");
      return PG_ERR_NOMEM;
    }
    O->dl.cap = bytes;
  }
  if (!O->dl_packed && (cudaEventCreateWithFlags(&O->dl_packed, cudaEventDisableTiming) != cudaSuccess ||
                        cudaEventCreateWithFlags(&O->dl_done, cudaEventDisableTiming) != cudaSuccess)) {
    set_last_error("pg_download_async: events");
    return PG_ERR_CUDA;
  }
  std::vector<size_t> off;
  for (PackSeg& s : segs) {
    bool is_float = false;
    off.push_back((uintptr_t)s.dst);
    if (bind_sources(S, s, is_float)) {
      set_last_error("pg_download_async: state array missing");
      return PG_ERR_INVALID;
    }
    s.dst = O->dl.dev + (uintptr_t)s.dst;
    launch_pack(s, S->g, is_float, S->stream);
  }
  cudaEventRecord(O->dl_packed, S->stream);
  cudaStreamWaitEvent(O->copy, O->dl_packed, 0);
  for (size_t m = 0; m < segs.size(); m++) {
    const size_t len = (size_t)segs[m].n[0] * segs[m].n[1] * segs[m].n[2] * sizeof(double);
    cudaMemcpyAsync(dst[m], O->dl.dev + off[m], len, cudaMemcpyDeviceToHost, O->copy);
  }
  cudaEventRecord(O->dl_done, O->copy);
  if (cudaGetLastError() != cudaSuccess) {
    set_last_error("pg_download_async: launch or copy");
    return PG_ERR_CUDA;
  }
  O->dl_pending = true;
  return PG_OK;
}

extern "C" int pg_download_wait(pg_solver* h) {
  if (!h) {
    set_last_error("pg_download_wait: null argument");
    return PG_ERR_INVALID;
  }
  OutputState* O = (OutputState*)h->S.out;
  if (!O || !O->dl_pending) return PG_OK;
  O->dl_pending = false;
  if (cudaEventSynchronize(O->dl_done) != cudaSuccess) {
    set_last_error("pg_download_wait: copy failed");
    return PG_ERR_CUDA;
  }
  return PG_OK;
}
