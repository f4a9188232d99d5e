// tlq_output.cu -- the output path (source/HydroCore.f90:253-395, `output`):
// UPrim of the current state in the reference's BIN, DAT or VTK format,
// without stalling the step loop.  The primitive snapshot is formed on the
// device behind the queued steps, copied to a page-locked host buffer on a
// copy stream (overlapping the steps that follow), and written to the file by
// a host thread.  One output is in flight at a time; the next call (or
// tlq_output_wait) waits for it.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "tlq_ctx.h"

namespace {

// Fortran Ew.d / Ew.dEe edit descriptor (gfortran's form: optional leading
// zero, exponent letter dropped when a 2-digit field overflows).
std::string fortran_e(double v, int w, int d, int e_digits) {
  std::string s;
  if (std::isnan(v)) {
    s = "NaN";
  } else if (std::isinf(v)) {
    s = v < 0 ? "-Infinity" : "Infinity";
  } else {
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.*e", d - 1, v);  // d significant digits, correctly rounded
    const char* p = buf;
    bool neg = false;
    if (*p == '-') {
      neg = true;
      ++p;
    }
    std::string digits;
    digits += p[0];
    const char* q = p + 1;
    if (*q == '.') ++q;
    while (*q && *q != 'e') digits += *q++;
    int ex = (*q == 'e') ? std::atoi(q + 1) : 0;
    if (v != 0.0) ex += 1;  // 0.ddd x 10^(ex+1)
    char eb[16];
    const int aex = ex < 0 ? -ex : ex;
    if (e_digits > 0) {
      std::snprintf(eb, sizeof eb, "E%c%0*d", ex < 0 ? '-' : '+', e_digits, aex);
    } else if (aex <= 99) {
      std::snprintf(eb, sizeof eb, "E%c%02d", ex < 0 ? '-' : '+', aex);
    } else {
      std::snprintf(eb, sizeof eb, "%c%03d", ex < 0 ? '-' : '+', aex);
    }
    s = std::string(neg ? "-" : "") + "0." + digits + eb;
  }
  if ((int)s.size() > w) return std::string(w, '*');
  return std::string(w - s.size(), ' ') + s;
}

std::string i_pad(int v, int w) {  // Iw.w (zero-padded), asterisks on overflow
  char b[32];
  std::snprintf(b, sizeof b, "%0*d", w, v);
  std::string s(b);
  if ((int)s.size() > w || v < 0) return std::string(w, '*');
  return s;
}

void put_be(FILE* f, double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  unsigned char b[8];
  for (int q = 0; q < 8; ++q) b[q] = (unsigned char)(u >> (56 - 8 * q));
  std::fwrite(b, 1, 8, f);
}

// The writers, on the host array W (the reference layout, ghosts included).
int write_bin(const std::string& fn, const double* W, size_t n) {
  FILE* f = std::fopen(fn.c_str(), "wb");
  if (!f) return TLQ_ERR_ARG;
  const size_t w = std::fwrite(W, sizeof(double), n, f);  // little-endian hosts
  std::fclose(f);
  return w == n ? TLQ_OK : TLQ_ERR_ARG;
}

int write_dat(const std::string& fn, const double* W, const tlq_config& c, double dx, double dy, double dz) {
  FILE* f = std::fopen(fn.c_str(), "w");
  if (!f) return TLQ_ERR_ARG;
  const long long sx = 5, sy = sx * (c.nx + 4), sz = sy * (c.ny + 4);
  auto at = [&](int e, int i, int j, int k) { return W[e + sx * (i + 1) + sy * (j + 1) + sz * (k + 1)]; };
  std::string line;
  // source/HydroCore.f90:296-302: k runs over the x range and i over the
  // z range (the reference's own loop bounds; the caller checked they stay
  // inside the array)
  for (int k = 1; k <= c.nx; ++k)
    for (int j = 1; j <= c.ny; ++j)
      for (int i = 1; i <= c.nz; ++i) {
        line.clear();
        line += fortran_e((double)i * dx, 16, 7, 3);
        line += fortran_e((double)j * dy, 16, 7, 3);
        line += fortran_e((double)k * dz, 16, 7, 3);
        for (int e = 0; e < 5; ++e) line += fortran_e(at(e, i, j, k), 16, 7, 3);
        line += '\n';
        std::fwrite(line.data(), 1, line.size(), f);
      }
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  return ok ? TLQ_OK : TLQ_ERR_ARG;
}

int write_vtk(const std::string& fn, const double* W, const tlq_config& c, double dx, double dy, double dz) {
  FILE* f = std::fopen(fn.c_str(), "wb");
  if (!f) return TLQ_ERR_ARG;
  auto text = [&](const std::string& s) { std::fwrite(s.data(), 1, s.size(), f); };
  char b[256];
  text("# vtk DataFile Version 2.0\n");
  text("output from Diable\n");
  text("BINARY\n");
  text("DATASET STRUCTURED_POINTS\n");
  std::snprintf(b, sizeof b, "DIMENSIONS %6d%6d%6d\n", c.nx, c.ny, c.nz);
  text(b);
  text("ORIGIN " + fortran_e(c.xl, 15, 7, 0) + fortran_e(c.yl, 15, 7, 0) + fortran_e(c.zl, 15, 7, 0) + "\n");
  text("SPACING" + fortran_e(dx, 15, 7, 0) + fortran_e(dy, 15, 7, 0) + fortran_e(dz, 15, 7, 0) + "\n");
  std::snprintf(b, sizeof b, "POINT_DATA %10lld\n", (long long)c.nx * c.ny * c.nz);
  text(b);
  const long long sx = 5, sy = sx * (c.nx + 4), sz = sy * (c.ny + 4);
  auto at = [&](int e, int i, int j, int k) { return W[e + sx * (i + 1) + sy * (j + 1) + sz * (k + 1)]; };
  text("SCALARS Density double 1\n");
  text("LOOKUP_TABLE default\n");
  for (int k = 1; k <= c.nz; ++k)
    for (int j = 1; j <= c.ny; ++j)
      for (int i = 1; i <= c.nx; ++i) put_be(f, at(0, i, j, k));
  text("\n");
  text("SCALARS Pressure double 1\n");
  text("LOOKUP_TABLE default\n");
  for (int k = 1; k <= c.nz; ++k)
    for (int j = 1; j <= c.ny; ++j)
      for (int i = 1; i <= c.nx; ++i) put_be(f, at(4, i, j, k));
  text("\n");
  text("VECTORS Velocity double\n");
  for (int k = 1; k <= c.nz; ++k)
    for (int j = 1; j <= c.ny; ++j)
      for (int i = 1; i <= c.nx; ++i) {
        put_be(f, at(1, i, j, k));
        put_be(f, at(2, i, j, k));
        put_be(f, at(3, i, j, k));
      }
  text("\n");
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  return ok ? TLQ_OK : TLQ_ERR_ARG;
}

}  // namespace

void output_join(tlq_ctx* ctx) {
  if (ctx->out_thread.joinable()) ctx->out_thread.join();
}

void output_free(tlq_ctx* ctx) {
  output_join(ctx);
  cudaFree(ctx->out_dev);
  cudaFreeHost(ctx->out_host);
  if (ctx->out_stream) cudaStreamDestroy(ctx->out_stream);
  for (int q = 0; q < 2; ++q)
    if (ctx->out_ev[q]) cudaEventDestroy(ctx->out_ev[q]);
  ctx->out_dev = nullptr;
  ctx->out_host = nullptr;
  ctx->out_stream = nullptr;
}

extern "C" {

int tlq_output(tlq_ctx* ctx, int format, const char* outputpath, int nout, int rank) {
  if (!ctx || !outputpath || nout < 0 || rank < 0) return TLQ_ERR_ARG;
  if (format != TLQ_OUT_DAT && format != TLQ_OUT_VTK && format != TLQ_OUT_BIN) return TLQ_ERR_ARG;
  if (!ctx->uploaded) {
    ctx->err = "tlq_output before tlq_upload";
    return TLQ_ERR_STATE;
  }
  const tlq_config& c = ctx->cfg;
  if (format == TLQ_OUT_DAT && (c.nz > c.nx + 2 || c.nx > c.nz + 2)) {
    // the reference's DAT loop (i over 1..nz indexing x, k over 1..nx
    // indexing z, HydroCore.f90:296-302) would leave the array
    ctx->err = "DAT output needs |nx - nz| <= 2 (the reference's loop bounds)";
    return TLQ_ERR_ARG;
  }
  // one output in flight: wait for the previous one and report its error
  output_join(ctx);
  if (ctx->out_rc != TLQ_OK) {
    const int rc = ctx->out_rc;
    ctx->out_rc = TLQ_OK;
    return rc;
  }
  const size_t n = (size_t)5 * (c.nx + 4) * (c.ny + 4) * (c.nz + 4);
  if (!ctx->out_dev) {
    if (cudaMalloc(&ctx->out_dev, n * sizeof(double)) != cudaSuccess ||
        cudaHostAlloc(&ctx->out_host, n * sizeof(double), cudaHostAllocDefault) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->out_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->out_ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->out_ev[1], cudaEventDisableTiming) != cudaSuccess) {
      output_free(ctx);
      ctx->err = "cannot allocate the output buffers";
      return TLQ_ERR_NOMEM;
    }
  }
  // snapshot behind the queued steps (the buffer parity read on the device)
  const bool carried = c.cooling != TLQ_COOL_NONE && c.precision == TLQ_PREC_FP64;
  cudaError_t e = launch_prims_soa_to_aos_clocked(ctx->P, ctx->A, ctx->L, ctx->U[0], ctx->U[1], ctx->clk,
                                                  ctx->it_base, carried ? ctx->Pc : nullptr, ctx->out_dev,
                                                  ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->out_ev[0], ctx->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->out_stream, ctx->out_ev[0], 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(ctx->out_host, ctx->out_dev, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->out_stream);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->out_ev[1], ctx->out_stream);
  if (e != cudaSuccess) {
    ctx->err = std::string("output snapshot: ") + cudaGetErrorString(e);
    return TLQ_ERR_CUDA;
  }
  // file names of HydroCore.f90:269-271
  const std::string base = std::string(outputpath);
  const std::string tag = i_pad(rank, 3) + "N" + i_pad(nout, 3);
  std::string fn;
  if (format == TLQ_OUT_BIN) fn = base + "points" + tag + ".bin";
  if (format == TLQ_OUT_DAT) fn = base + "points" + tag + ".dat";
  if (format == TLQ_OUT_VTK) fn = base + "EPV" + tag + ".vtk";
  const double dx = ctx->P.dx, dy = ctx->P.dy, dz = ctx->P.dz;
  const double* W = ctx->out_host;
  cudaEvent_t done = ctx->out_ev[1];
  const tlq_config cfg = c;
  int device = 0;
  cudaGetDevice(&device);
  ctx->out_thread = std::thread([ctx, fn, W, n, cfg, dx, dy, dz, format, done, device]() {
    cudaSetDevice(device);
    if (cudaEventSynchronize(done) != cudaSuccess) {
      ctx->out_rc = TLQ_ERR_CUDA;
      return;
    }
    int rc = TLQ_OK;
    if (format == TLQ_OUT_BIN) rc = write_bin(fn, W, n);
    if (format == TLQ_OUT_DAT) rc = write_dat(fn, W, cfg, dx, dy, dz);
    if (format == TLQ_OUT_VTK) rc = write_vtk(fn, W, cfg, dx, dy, dz);
    ctx->out_rc = rc;
  });
  return TLQ_OK;
}

int tlq_output_wait(tlq_ctx* ctx) {
  if (!ctx) return TLQ_ERR_ARG;
  output_join(ctx);
  const int rc = ctx->out_rc;
  ctx->out_rc = TLQ_OK;
  if (rc != TLQ_OK) ctx->err = "output: writing the file failed";
  return rc;
}

}  // extern "C"
