// Domain decomposition (include/mom5gpu.h, "domain decomposition"): a block of a
// 2-D layout is a non-cyclic mom5gpu_domain whose halos facing other blocks are
// filled by exchanges between the phases of a step, where the reference calls
// mpp_update_domains (ocean_tracer_advect.F90:3912, :3970; ocean_model.F90:
// 1903-1911; ocean_barotropic.F90:3383, :2846-2901).  This file holds the halo
// geometry (pure host arithmetic, shared by one-GPU and multi-process callers),
// the strip buffers of the MDFL intermediates, the box-copy kernel the
// exchanges use on one GPU, and the phase entry points.
#include <string.h>

#include <vector>

#include "internal.h"

using namespace mom5;

namespace {

// A one-cell halo region of a data-domain array of nlev levels (level stride
// (ni+2)(nj+2)): SEND = the compute cells next to `side`, RECV = the halo cells
// on `side`.  Faces span the compute rows or columns, corners are one cell.
void field_region(const mom5gpu_dims& dm, int nlev, int side, int role, long* off, long st[3], int n[3]) {
  const long nxd = dm.ni + 2, n2 = nxd * (dm.nj + 2);
  const bool send = role == MOM5GPU_SEND;
  int i0 = 1, j0 = 1, ni = 1, nj = 1;
  switch (side) {
    case MOM5GPU_WEST: i0 = send ? 1 : 0; nj = dm.nj; break;
    case MOM5GPU_EAST: i0 = send ? dm.ni : dm.ni + 1; nj = dm.nj; break;
    case MOM5GPU_SOUTH: j0 = send ? 1 : 0; ni = dm.ni; break;
    case MOM5GPU_NORTH: j0 = send ? dm.nj : dm.nj + 1; ni = dm.ni; break;
    case MOM5GPU_SOUTHWEST: i0 = send ? 1 : 0; j0 = send ? 1 : 0; break;
    case MOM5GPU_SOUTHEAST: i0 = send ? dm.ni : dm.ni + 1; j0 = send ? 1 : 0; break;
    case MOM5GPU_NORTHWEST: i0 = send ? 1 : 0; j0 = send ? dm.nj : dm.nj + 1; break;
    default: i0 = send ? dm.ni : dm.ni + 1; j0 = send ? dm.nj : dm.nj + 1; break;
  }
  *off = (long)j0 * nxd + i0;
  st[0] = 1;
  st[1] = nxd;
  st[2] = n2;
  n[0] = ni;
  n[1] = nj;
  n[2] = nlev;
}

// The boxes of one launch travel in the launch's own parameter block, by value:
// no table is uploaded, so the launch needs no copy engine (those stay with the
// host link, where a small upload would queue behind gigabytes of field copies)
// and the host never waits for an earlier launch to free a table.
template <int N>
struct BoxSet {
  mom5gpu_box b[N];
};
constexpr int kBoxesSmall = 8, kBoxesPerLaunch = 256;  // 640 B and 20 KB of parameters
static_assert(sizeof(BoxSet<kBoxesPerLaunch>) <= 32000, "kernel parameters are limited to 32764 bytes");

template <int N>
__global__ void k_copy_boxes(const __grid_constant__ BoxSet<N> set) {
  const mom5gpu_box& b = set.b[blockIdx.y];
  const long nx = b.n[0], nxy = nx * b.n[1], total = nxy * b.n[2];
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long z = e / nxy, r = e - z * nxy, y = r / nx, x = r - y * nx;
    b.dst[x * b.dst_stride[0] + y * b.dst_stride[1] + z * b.dst_stride[2]] =
        b.src[x * b.src_stride[0] + y * b.src_stride[1] + z * b.src_stride[2]];
  }
}

template <int N>
cudaError_t launch_boxes(const mom5gpu_box* boxes, int nb, long most, cudaStream_t s) {
  BoxSet<N> set;
  memset(&set, 0, sizeof(set));
  memcpy(set.b, boxes, sizeof(mom5gpu_box) * nb);
  unsigned bx = (unsigned)((most + 255) / 256);
  if (bx > 1024) bx = 1024;
  k_copy_boxes<N><<<dim3(bx, nb), 256, 0, s>>>(set);
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int mom5gpu_halo_region(const mom5gpu_dims* dims, int kind, int nlev, int side, int role, long* offset,
                        long stride[3], int n[3]) {
  if (!dims || !offset || !stride || !n || side < 0 || side > 7 || (role != MOM5GPU_SEND && role != MOM5GPU_RECV))
    return MOM5GPU_EINVAL;
  const mom5gpu_dims& dm = *dims;
  if (dm.ni < 2 || dm.nj < 2 || dm.nk < 1) return MOM5GPU_EINVAL;
  const long nxd = dm.ni + 2, n2 = nxd * (dm.nj + 2);
  const long ntr = dm.num_prog_tracers > 0 ? dm.num_prog_tracers : 1;
  const bool send = role == MOM5GPU_SEND;
  switch (kind) {
    case MOM5GPU_HALO_FIELD:
      if (nlev < 1) return MOM5GPU_EINVAL;
      field_region(dm, nlev, side, role, offset, stride, n);
      return MOM5GPU_OK;
    case MOM5GPU_HALO_BT_ETA:
    case MOM5GPU_HALO_BT_PS:
      field_region(dm, 1, side, role, offset, stride, n);
      return MOM5GPU_OK;
    case MOM5GPU_HALO_MDFL_Z: {
      // SEND: tracer_mdfl columns 1,2 (west) or ni-1,ni (east), rows 1..nj, every
      // (tracer, level) plane; RECV: strip slots 0,1 (i = -1, 0) or 2,3 (ni+1, ni+2)
      if (side != MOM5GPU_WEST && side != MOM5GPU_EAST) return MOM5GPU_EINVAL;
      n[0] = 2;
      n[1] = dm.nj;
      n[2] = (int)(ntr * dm.nk);
      if (send) {
        *offset = nxd + (side == MOM5GPU_WEST ? 1 : dm.ni - 1);
        stride[0] = 1;
        stride[1] = nxd;
        stride[2] = n2;
      } else {
        *offset = side == MOM5GPU_WEST ? 0 : 2;
        stride[0] = 1;
        stride[1] = 4;
        stride[2] = 4L * dm.nj;
      }
      return MOM5GPU_OK;
    }
    case MOM5GPU_HALO_MDFL_X: {
      // SEND: rows 1,2 (south) or nj-1,nj (north), columns 1..ni; RECV: strip
      // slots 0,1 (j = -1, 0) or 2,3 (nj+1, nj+2)
      if (side != MOM5GPU_SOUTH && side != MOM5GPU_NORTH) return MOM5GPU_EINVAL;
      n[0] = dm.ni;
      n[1] = 2;
      n[2] = (int)(ntr * dm.nk);
      if (send) {
        *offset = (side == MOM5GPU_SOUTH ? 1 : dm.nj - 1) * nxd + 1;
        stride[0] = 1;
        stride[1] = nxd;
        stride[2] = n2;
      } else {
        *offset = (side == MOM5GPU_SOUTH ? 0 : 2) * (long)dm.ni;
        stride[0] = 1;
        stride[1] = dm.ni;
        stride[2] = 4L * dm.ni;
      }
      return MOM5GPU_OK;
    }
    default:
      return MOM5GPU_EINVAL;
  }
}

int mom5gpu_set_neighbours(mom5gpu_domain* d, int west, int east, int south, int north) {
  if (!d) return MOM5GPU_EINVAL;
  const Geo& g = d->geo;
  if ((west || east) && g.cx) return fail(d, MOM5GPU_EINVAL, "set_neighbours: a block is created non-cyclic");
  if ((south || north) && g.cy) return fail(d, MOM5GPU_EINVAL, "set_neighbours: a block is created non-cyclic");
  if (g.ni < 2 || g.nj < 2) return fail(d, MOM5GPU_EINVAL, "set_neighbours: a block needs ni, nj >= 2");
  if (d->dims.num_prog_tracers > kMdflChunk)
    return fail(d, MOM5GPU_EUNSUPPORTED, "decomposed stepping advects at most %d tracers", kMdflChunk);
  int nbr = (west ? 1 : 0) | (east ? 2 : 0) | (south ? 4 : 0) | (north ? 8 : 0);
  const size_t ntr = d->dims.num_prog_tracers > 0 ? d->dims.num_prog_tracers : 1;
  if (!d->hz) {
    size_t bz = sizeof(double) * ntr * g.nk * g.nj * 4, bx = sizeof(double) * ntr * g.nk * 4 * g.ni;
    cudaError_t e = cudaMalloc(&d->hz, bz);
    if (e == cudaSuccess) e = cudaMalloc(&d->hx, bx);
    if (e == cudaSuccess) e = cudaMemset(d->hz, 0, bz);
    if (e == cudaSuccess) e = cudaMemset(d->hx, 0, bx);
    if (e != cudaSuccess) {
      if (d->hz) cudaFree(d->hz);
      if (d->hx) cudaFree(d->hx);
      d->hz = d->hx = nullptr;
      return cuda_fail(d, e, "set_neighbours: halo strips");
    }
    d->bytes += bz + bx;
  }
  d->nbr = nbr;
  return MOM5GPU_OK;
}

int mom5gpu_set_mask_halo2(mom5gpu_domain* d, const double* tmask_halo2) {
  if (!d || !tmask_halo2) return d ? fail(d, MOM5GPU_EINVAL, "set_mask_halo2: null mask") : MOM5GPU_EINVAL;
  if (!d->advect_ready || !d->mask2)
    return fail(d, MOM5GPU_ESTATE, "set_mask_halo2 before mom5gpu_tracer_advect_init");
  const Geo& g = d->geo;
  const size_t cnt = (size_t)(g.ni + 4) * (g.nj + 4) * g.nk;
  std::vector<uint8_t> m(cnt);
  for (size_t q = 0; q < cnt; ++q) {
    double v = tmask_halo2[q];
    if (v != 0.0 && v != 1.0) return fail(d, MOM5GPU_EINVAL, "set_mask_halo2: values must be 0 or 1");
    m[q] = v != 0.0;
  }
  cudaError_t e = cudaMemcpy(d->mask2, m.data(), cnt, cudaMemcpyHostToDevice);
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "set_mask_halo2");
}

int mom5gpu_halo_base(mom5gpu_domain* d, int kind, int field, int n, int level, int role, double** base) {
  if (!d || !base) return MOM5GPU_EINVAL;
  const bool send = role == MOM5GPU_SEND;
  switch (kind) {
    case MOM5GPU_HALO_FIELD: {
      double* p = fptr(d, field, n == 0 && field == MOM5GPU_TRACER ? 1 : n, level);
      if (!p) return fail(d, MOM5GPU_EINVAL, "halo_base: field %d (n %d, level %d)", field, n, level);
      *base = p;
      return MOM5GPU_OK;
    }
    case MOM5GPU_HALO_MDFL_Z:
      if (!(send ? d->mdfl_a : d->hz)) return fail(d, MOM5GPU_ESTATE, "halo_base: MDFL scratch or strips not set up");
      *base = send ? d->mdfl_a : d->hz;
      return MOM5GPU_OK;
    case MOM5GPU_HALO_MDFL_X:
      if (!(send ? d->mdfl_b : d->hx)) return fail(d, MOM5GPU_ESTATE, "halo_base: MDFL scratch or strips not set up");
      *base = send ? d->mdfl_b : d->hx;
      return MOM5GPU_OK;
    case MOM5GPU_HALO_BT_ETA:
    case MOM5GPU_HALO_BT_PS:
      if (!d->bt || !d->baro_ready) return fail(d, MOM5GPU_ESTATE, "halo_base: barotropic step not initialised");
      if (kind == MOM5GPU_HALO_BT_ETA && level != 0 && level != 1)
        return fail(d, MOM5GPU_EINVAL, "halo_base: eta plane %d (0 or 1)", level);
      *base = kind == MOM5GPU_HALO_BT_ETA ? d->bt + (size_t)level * d->geo.n2 : d->bt + 7 * (size_t)d->geo.n2;
      return MOM5GPU_OK;
    default:
      return fail(d, MOM5GPU_EINVAL, "halo_base: kind %d", kind);
  }
}

int mom5gpu_copy_boxes(const mom5gpu_box* boxes, int count, void* stream) {
  if (count < 0 || (count > 0 && !boxes)) return MOM5GPU_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  for (int b0 = 0; b0 < count; b0 += kBoxesPerLaunch) {
    int nb = count - b0 < kBoxesPerLaunch ? count - b0 : kBoxesPerLaunch;
    long most = 1;
    for (int b = 0; b < nb; ++b) {
      const mom5gpu_box& x = boxes[b0 + b];
      if (!x.src || !x.dst || x.n[0] < 0 || x.n[1] < 0 || x.n[2] < 0)
        return fail(nullptr, MOM5GPU_EINVAL, "copy_boxes: box %d has a null pointer or a negative extent", b0 + b);
      long e = (long)x.n[0] * x.n[1] * x.n[2];
      if (e > most) most = e;
    }
    cudaError_t e = nb <= kBoxesSmall ? launch_boxes<kBoxesSmall>(boxes + b0, nb, most, s)
                                      : launch_boxes<kBoxesPerLaunch>(boxes + b0, nb, most, s);
    if (e != cudaSuccess) return fail(nullptr, MOM5GPU_ECUDA, "copy_boxes: %s", cudaGetErrorString(e));
  }
  return MOM5GPU_OK;
}

int mom5gpu_mdfl_pass(mom5gpu_domain* d, int pass, int taum1, int tau, double dtime) {
  if (!d) return MOM5GPU_EINVAL;
  if (pass < 1 || pass > 3) return fail(d, MOM5GPU_EINVAL, "mdfl_pass: pass %d (1 z, 2 x, 3 y)", pass);
  if (taum1 < 1 || taum1 > 3 || tau < 1 || tau > 3) return fail(d, MOM5GPU_EINVAL, "mdfl_pass: time levels");
  if (!d->advect_ready) return fail(d, MOM5GPU_ESTATE, "mdfl_pass before mom5gpu_tracer_advect_init");
  const int ntr = d->dims.num_prog_tracers;
  if (ntr == 0) return MOM5GPU_OK;
  if (ntr > kMdflChunk) return fail(d, MOM5GPU_EUNSUPPORTED, "mdfl_pass: at most %d tracers", kMdflChunk);
  if (d->opt.precision != MOM5GPU_PRECISION_FP64) return fail(d, MOM5GPU_EUNSUPPORTED, "mdfl_pass: FP64 only");
  int sweby = -1;
  for (int n = 0; n < ntr; ++n) {
    int h = d->scheme[n].horz;
    int s = h == MOM5GPU_ADVECT_MDFL_SWEBY ? 1 : h == MOM5GPU_ADVECT_DST_LINEAR ? 0 : -1;
    if (s < 0 || (sweby >= 0 && s != sweby))
      return fail(d, MOM5GPU_EUNSUPPORTED, "mdfl_pass: every tracer on MDFL Sweby, or every one on DST linear");
    sweby = s;
  }
  if (d->opt.zero_tracer_advect_horz) return fail(d, MOM5GPU_EUNSUPPORTED, "mdfl_pass: zero_tracer_advect_horz");
  int rc = ensure_mdfl_scratch(d, ntr);
  if (rc) return rc;
  if (pass == 1) {
    double* th = fptr(d, MOM5GPU_TH_TENDENCY, 1, 0);
    if (!th) return MOM5GPU_ENOMEM;
    launch_zero_ring(d->geo, th, (long)ntr * d->geo.nk, d->stream);
    count_launches(d, 1);
  }
  ClockScope clk(d, SEC_MDFL);
  MdflArgs a;
  if ((rc = make_mdfl_args(d, 1, ntr, taum1, tau, dtime, &a))) return rc;
  a.th_fresh = 1;
  run_mdfl_pass(a, d->opt.advect_sweby_all != 0, sweby == 1, pass, d->stream);
  count_launches(d, 1);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MOM5GPU_OK : cuda_fail(d, e, "mdfl_pass");
}

int mom5gpu_barotropic_phase(mom5gpu_domain* d, int tau, int taup1, int phase, int itime) {
  if (!d) return MOM5GPU_EINVAL;
  if (tau < 1 || tau > 3 || taup1 < 1 || taup1 > 3) return fail(d, MOM5GPU_EINVAL, "barotropic_phase: time levels");
  return launch_barotropic_phase(d, tau, taup1, phase, itime);
}

}  // extern "C"
