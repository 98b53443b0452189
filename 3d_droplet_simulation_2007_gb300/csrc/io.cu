// io.cu -- snapshots and the reference's output/restart files (host side).
//
// A snapshot copies the pressure, velocity and volume fraction device to
// device (one pass over HBM, on the context stream, so it is ordered after
// the step that produced them) and then to pinned host memory on a separate
// copy stream: the next time steps run while the host copy is in flight.
// The writers format the last snapshot:
//  * printtecp (main.f:5105-5153): main####.plt, Tecplot ASCII of X, Y, Z, U,
//    V, W, CC at the cell nodes, velocities averaged to the cell centre;
//  * the pressure slice of printout (main.f:5074-5095): pressure####.plt, the
//    mid-z plane of p / tauh^2 * rho1_SI;
//  * savedata / iniget (main.f:5414-5467, 698-790): the unformatted restart
//    file.  The reference's savedata opens unit 3 but writes unit 2, so its
//    file cannot be read back by iniget; here both use the same file and the
//    record layout iniget reads (gfortran sequential records: a 4-byte length
//    before and after every record).
// Number formats follow the Fortran edit descriptors: E15.7 after one blank
// for the data lines; list-directed output (a leading blank, default
// integers in 12 columns) for the headers.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "dsg_internal.cuh"

namespace {

const int kSnapFields[dsg_ctx::kSnapFields] = {DSG_F_P, DSG_F_U, DSG_F_V, DSG_F_W, DSG_F_CC};

int snap_slot(int field) {
  for (int s = 0; s < dsg_ctx::kSnapFields; s++)
    if (kSnapFields[s] == field) return s;
  return -1;
}

// Fortran Ew.d with w = 15, d = 7: [-]0.dddddddE+ee (E dropped for a
// three-digit exponent), right-justified.
void fort_e15_7(char *out, double x) {
  char buf[64];
  if (isnan(x)) {
    snprintf(out, 16, "%15s", "NaN");
    return;
  }
  if (isinf(x)) {
    snprintf(out, 16, "%15s", x > 0 ? "Infinity" : "-Infinity");
    return;
  }
  if (x == 0.0) {
    snprintf(out, 16, "%15s", "0.0000000E+00");
    return;
  }
  snprintf(buf, sizeof buf, "%.6E", x);  // [-]d.ddddddE[+-]xx: 7 significant digits
  const bool neg = buf[0] == '-';
  const char *m = buf + (neg ? 1 : 0);
  const char *e = strchr(m, 'E');
  const int ex = atoi(e + 1) + 1;  // 0.d form
  char digits[8];
  digits[0] = m[0];
  memcpy(digits + 1, m + 2, 6);
  digits[7] = 0;
  char mant[32];
  const int ax = ex < 0 ? -ex : ex;
  if (ax <= 99)
    snprintf(mant, sizeof mant, "%s0.%sE%c%02d", neg ? "-" : "", digits, ex < 0 ? '-' : '+', ax);
  else
    snprintf(mant, sizeof mant, "%s0.%s%c%03d", neg ? "-" : "", digits, ex < 0 ? '-' : '+', ax);
  snprintf(out, 16, "%15.15s", mant);  // E15.7 fields hold at most 14 characters
}

void put_row(FILE *f, const double *v, int n) {
  char cell[16];
  for (int q = 0; q < n; q++) {
    fort_e15_7(cell, v[q]);
    fputc(' ', f);
    fputs(cell, f);
  }
  fputc('\n', f);
}

// gfortran sequential unformatted record
bool put_rec(FILE *f, const void *p, int32_t n) {
  return fwrite(&n, 4, 1, f) == 1 && fwrite(p, 1, (size_t)n, f) == (size_t)n && fwrite(&n, 4, 1, f) == 1;
}

bool get_rec(FILE *f, void *p, int32_t n) {
  int32_t a = 0, b = 0;
  if (fread(&a, 4, 1, f) != 1 || a != n) return false;
  if (fread(p, 1, (size_t)n, f) != (size_t)n) return false;
  return fread(&b, 4, 1, f) == 1 && b == n;
}

int alloc_snapshot(dsg_ctx *ctx) {
  if (ctx->snap_dev) return DSG_OK;
  const size_t n = ctx->fine().count();
  DSG_CK(ctx, cudaMalloc(&ctx->snap_dev, dsg_ctx::kSnapFields * n * sizeof(double)));
  DSG_CK(ctx, cudaMallocHost(&ctx->snap_host, dsg_ctx::kSnapFields * n * sizeof(double)));
  DSG_CK(ctx, cudaStreamCreateWithFlags(&ctx->snap_stream, cudaStreamNonBlocking));
  DSG_CK(ctx, cudaEventCreateWithFlags(&ctx->snap_ready, cudaEventDisableTiming));
  DSG_CK(ctx, cudaEventCreateWithFlags(&ctx->snap_done, cudaEventDisableTiming));
  return DSG_OK;
}

// The last snapshot on the host (taking one now if there is none).
int snapshot_host(dsg_ctx *ctx, const double **host, int *t) {
  if (!ctx->snap_pending && ctx->snap_t < 0) {
    int rc = dsg_snapshot(ctx, 0);
    if (rc) return rc;
  }
  int rc = dsg_snapshot_wait(ctx, t);
  if (rc) return rc;
  *host = ctx->snap_host;
  return DSG_OK;
}

}  // namespace

namespace dsg {
void snapshot_release(dsg_ctx *ctx) {
  if (ctx->snap_stream) cudaStreamSynchronize(ctx->snap_stream);
  if (ctx->snap_ready) cudaEventDestroy(ctx->snap_ready);
  if (ctx->snap_done) cudaEventDestroy(ctx->snap_done);
  if (ctx->snap_stream) cudaStreamDestroy(ctx->snap_stream);
  if (ctx->snap_dev) cudaFree(ctx->snap_dev);
  if (ctx->snap_host) cudaFreeHost(ctx->snap_host);
  ctx->snap_ready = ctx->snap_done = nullptr;
  ctx->snap_stream = nullptr;
  ctx->snap_dev = nullptr;
  ctx->snap_host = nullptr;
}
}  // namespace dsg

extern "C" {

int dsg_snapshot(dsg_ctx *ctx, int t) {
  if (!ctx) return DSG_E_ARG;
  int rc = alloc_snapshot(ctx);
  if (rc) return rc;
  if (ctx->snap_pending) DSG_CK(ctx, cudaEventSynchronize(ctx->snap_done));  // one copy in flight at a time
  const size_t n = ctx->fine().count();
  for (int s = 0; s < dsg_ctx::kSnapFields; s++)
    DSG_CK(ctx, cudaMemcpyAsync(ctx->snap_dev + s * n, ctx->f[kSnapFields[s]], n * sizeof(double),
                                cudaMemcpyDeviceToDevice, ctx->stream));
  DSG_CK(ctx, cudaEventRecord(ctx->snap_ready, ctx->stream));
  DSG_CK(ctx, cudaStreamWaitEvent(ctx->snap_stream, ctx->snap_ready, 0));
  DSG_CK(ctx, cudaMemcpyAsync(ctx->snap_host, ctx->snap_dev, dsg_ctx::kSnapFields * n * sizeof(double),
                              cudaMemcpyDeviceToHost, ctx->snap_stream));
  DSG_CK(ctx, cudaEventRecord(ctx->snap_done, ctx->snap_stream));
  ctx->snap_pending = true;
  ctx->snap_t = t;
  return DSG_OK;
}

int dsg_snapshot_wait(dsg_ctx *ctx, int *t) {
  if (!ctx) return DSG_E_ARG;
  if (ctx->snap_t < 0) return dsg::set_error(ctx, DSG_E_STATE, "no snapshot taken");
  if (ctx->snap_pending) {
    DSG_CK(ctx, cudaEventSynchronize(ctx->snap_done));
    ctx->snap_pending = false;
  }
  if (t) *t = ctx->snap_t;
  return DSG_OK;
}

int dsg_snapshot_field(dsg_ctx *ctx, int field, double *host) {
  if (!ctx || !host) return DSG_E_ARG;
  const int s = snap_slot(field);
  if (s < 0) return dsg::set_error(ctx, DSG_E_ARG, "field %d is not part of a snapshot (p, u, v, w, cc)", field);
  int rc = dsg_snapshot_wait(ctx, nullptr);
  if (rc) return rc;
  const size_t n = ctx->fine().count();
  memcpy(host, ctx->snap_host + s * n, n * sizeof(double));
  return DSG_OK;
}

int dsg_write_tecplot(dsg_ctx *ctx, const char *path) {
  if (!ctx || !path) return DSG_E_ARG;
  const double *H;
  int t;
  int rc = snapshot_host(ctx, &H, &t);
  if (rc) return rc;
  const size_t n = ctx->fine().count();
  const double *u = H + snap_slot(DSG_F_U) * n, *v = H + snap_slot(DSG_F_V) * n, *w = H + snap_slot(DSG_F_W) * n;
  const double *cc = H + snap_slot(DSG_F_CC) * n;
  const int nx = ctx->nx, ny = ctx->ny, nz = ctx->nz;
  const dsg::Dims d = ctx->fine();
  const double h = ctx->s.h, L = ctx->s.lengthscale;
  FILE *f = fopen(path, "w");
  if (!f) return dsg::set_error(ctx, DSG_E_ARG, "cannot open %s for writing", path);
  fprintf(f, " VARIABLES=\"X\",\"Y\",\"Z\",\"U\",\"V\",\"W\",\"CC\"\n");
  fprintf(f, " zone i=%12d j=%12d k=%12d\n", nx, ny - 1, nz);
  double row[7];
  for (int k = 1; k <= nz; k++) {
    const double zz = k * h * L * 1000;
    for (int j = 2; j <= ny; j++) {
      const double yy = j * h * L * 1000;
      for (int i = 1; i <= nx; i++) {
        const size_t q = d.ix(i, j, k);
        row[0] = i * h * L * 1000;
        row[1] = yy;
        row[2] = zz;
        row[3] = i == nx ? u[q] : .5 * (u[q] + u[q + 1]);
        row[4] = j == ny ? v[q] : .5 * (v[q] + v[q + d.sy()]);
        row[5] = k == nz ? w[q] : .5 * (w[q] + w[q + d.sz()]);
        row[6] = cc[q];
        put_row(f, row, 7);
      }
    }
  }
  const bool ok = fclose(f) == 0;
  return ok ? DSG_OK : dsg::set_error(ctx, DSG_E_ARG, "write error on %s", path);
}

int dsg_write_pressure_slice(dsg_ctx *ctx, const char *path) {
  if (!ctx || !path) return DSG_E_ARG;
  const double *H;
  int t;
  int rc = snapshot_host(ctx, &H, &t);
  if (rc) return rc;
  const size_t n = ctx->fine().count();
  const double *p = H + snap_slot(DSG_F_P) * n;
  const int nx = ctx->nx, ny = ctx->ny, nz = ctx->nz;
  const dsg::Dims d = ctx->fine();
  const double h = ctx->s.h, tauh = ctx->s.tauh, rho1 = ctx->cfg.rho1_si;
  FILE *f = fopen(path, "w");
  if (!f) return dsg::set_error(ctx, DSG_E_ARG, "cannot open %s for writing", path);
  fprintf(f, " VARIABLES=\"x\",\"y\",\"p\"\n");
  fprintf(f, " zone i=%12dj=%12d\n", nx - 2, ny - 2);
  const int k = (nz - 2) / 2;
  double row[3];
  for (int j = 2; j <= ny - 1; j++)
    for (int i = 2; i <= nx - 1; i++) {
      row[0] = h * i;
      row[1] = h * j;
      row[2] = p[d.ix(i, j, k)] / (tauh * tauh) * rho1;
      put_row(f, row, 3);
    }
  const bool ok = fclose(f) == 0;
  return ok ? DSG_OK : dsg::set_error(ctx, DSG_E_ARG, "write error on %s", path);
}

int dsg_savedata(dsg_ctx *ctx, const char *path, int t0) {
  if (!ctx || !path) return DSG_E_ARG;
  const double *H;
  int t;
  int rc = snapshot_host(ctx, &H, &t);
  if (rc) return rc;
  const dsg_config &c = ctx->cfg;
  FILE *f = fopen(path, "wb");
  if (!f) return dsg::set_error(ctx, DSG_E_ARG, "cannot open %s for writing", path);
  bool ok = true;
  auto I = [&](int32_t v) { ok = ok && put_rec(f, &v, 4); };
  auto D = [&](double v) { ok = ok && put_rec(f, &v, 8); };
  I(t0);
  I(c.nx), I(c.ny), I(c.nz), I(c.tmax), I(c.nfilter), I(c.cycles);
  D(c.omega);
  I(c.npre), I(c.ntop), I(c.npost), I(c.restart);
  D(c.maxcfl);
  I(c.iturb), I(c.convectype), I(c.hswitch);
  D(c.xvel1_si), D(c.yvel1_si), D(c.zvel1_si), D(c.xvel2_si), D(c.yvel2_si), D(c.zvel2_si);
  D(c.rho2_si), D(c.rho1_si), D(c.sigma_si), D(c.visc2_si), D(c.visc1_si), D(c.grav_si), D(c.grav1_si);
  I(c.icase), I(c.ibc);
  D(c.length_si), D(c.radius_si);
  I(c.tprint), I(c.ntecplot), I(c.tsave);
  const size_t n = ctx->fine().count();
  const double *u = H + snap_slot(DSG_F_U) * n, *v = H + snap_slot(DSG_F_V) * n, *w = H + snap_slot(DSG_F_W) * n;
  const double *cc = H + snap_slot(DSG_F_CC) * n;
  for (size_t q = 0; q < n && ok; q++) {  // k, j, i order = linear order
    const double r[4] = {u[q], v[q], w[q], cc[q]};
    ok = put_rec(f, r, 32);
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? DSG_OK : dsg::set_error(ctx, DSG_E_ARG, "write error on %s", path);
}

int dsg_iniget(dsg_ctx *ctx, const char *path, int *t0) {
  if (!ctx || !path) return DSG_E_ARG;
  FILE *f = fopen(path, "rb");
  if (!f) return dsg::set_error(ctx, DSG_E_ARG, "cannot open %s", path);
  bool ok = true;
  int32_t iv[4];
  double dv;
  auto I = [&](int32_t *v) { ok = ok && get_rec(f, v, 4); };
  auto D = [&]() { ok = ok && get_rec(f, &dv, 8); };
  int32_t tt = 0;
  I(&tt);
  I(&iv[0]), I(&iv[1]), I(&iv[2]);
  if (ok && (iv[0] != ctx->nx || iv[1] != ctx->ny || iv[2] != ctx->nz)) {
    fclose(f);
    return dsg::set_error(ctx, DSG_E_ARG, "%s holds a %dx%dx%d grid, the context %dx%dx%d", path, iv[0], iv[1], iv[2],
                          ctx->nx, ctx->ny, ctx->nz);
  }
  // the remaining parameters (main.f:708-747): read and checked for shape only;
  // the context keeps its own configuration
  for (int q = 0; q < 3; q++) I(&iv[3]);  // tmax, nfilter, cycles
  D();                                   // omega
  for (int q = 0; q < 4; q++) I(&iv[3]);  // npre, ntop, npost, restart
  D();                                   // maxcfl
  for (int q = 0; q < 3; q++) I(&iv[3]);  // iturb, convectype, hswitch
  for (int q = 0; q < 13; q++) D();       // velocities, densities, sigma, viscosities, gravities
  for (int q = 0; q < 2; q++) I(&iv[3]);  // icase, ibc
  for (int q = 0; q < 2; q++) D();        // length_SI, radius_si
  for (int q = 0; q < 3; q++) I(&iv[3]);  // tprint, ntecplot, tsave
  const size_t n = ctx->fine().count();
  std::vector<double> u(n), v(n), w(n), cc(n);
  for (size_t q = 0; q < n && ok; q++) {
    double r[4];
    ok = get_rec(f, r, 32);
    u[q] = r[0], v[q] = r[1], w[q] = r[2], cc[q] = r[3];
  }
  fclose(f);
  if (!ok) return dsg::set_error(ctx, DSG_E_ARG, "%s is not a restart file of this grid (bad record)", path);
  int rc = dsg_upload(ctx, DSG_F_U, u.data());
  if (!rc) rc = dsg_upload(ctx, DSG_F_V, v.data());
  if (!rc) rc = dsg_upload(ctx, DSG_F_W, w.data());
  if (!rc) rc = dsg_upload(ctx, DSG_F_CC, cc.data());
  if (!rc) rc = dsg::restart_state(ctx);
  if (rc) return rc;
  if (t0) *t0 = tt;
  return DSG_OK;
}

// printout's file schedule (main.f:5020-5104): main####.plt every ntecplot
// steps, pressure####.plt every 100 steps, the restart file at t = tsave.
// Files go to directory `dir` (NULL: the working directory).
int dsg_printout(dsg_ctx *ctx, int t, const char *dir) {
  if (!ctx) return DSG_E_ARG;
  const dsg_config &c = ctx->cfg;
  const bool tec = c.ntecplot > 0 && t % c.ntecplot == 0;
  const bool pre = t % 100 == 0;
  const bool sav = t == c.tsave;
  if (!tec && !pre && !sav) return DSG_OK;
  int rc = dsg_snapshot(ctx, t);
  if (rc) return rc;
  const std::string base = dir && *dir ? std::string(dir) + "/" : std::string();
  char name[64];
  if (tec) {
    snprintf(name, sizeof name, "main%04d.plt", t / c.ntecplot);
    rc = dsg_write_tecplot(ctx, (base + name).c_str());
    if (rc) return rc;
  }
  if (pre) {
    snprintf(name, sizeof name, "pressure%04d.plt", t / 100);
    rc = dsg_write_pressure_slice(ctx, (base + name).c_str());
    if (rc) return rc;
  }
  if (sav) rc = dsg_savedata(ctx, (base + "save.dat").c_str(), t);
  return rc;
}

}  // extern "C"
