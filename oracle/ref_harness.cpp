// ORACLE PIN — test infrastructure only, built only where the reference tree is
// mounted (oracle/build.py build_ref). It drives the reference's own
// header-only NanoVDB (nanovdb/NanoVDB.h, nanovdb/util/GridBuilder.h) on the
// host to produce golden vectors for tests/golden/: grids are built with
// nanovdb::GridBuilder, queried through nanovdb::ReadAccessor, and mutated
// through LeafNode::setValueOnly / the leaf value masks, and the bodies of the
// reference kernels are restated around those calls in float arithmetic:
//   density_forward_kernel      plenvdb/lib/vdb/densityvdb.cu:101-125
//   density_backward_kernel     densityvdb.cu:16-27, 143-167 (sequential adds)
//   color_forward_kernel        colorvdb.cu:16-26, 81-111
//   color_backward_kernel       colorvdb.cu:28-37, 130-160
//   density_updateData*         densityvdb.cu:185-330 (modes 0, 1, 2)
//   color_updateData*           colorvdb.cu:179-331
//   trigetDensity               renderer.cu:191-220 (index grid, int() truncation)
//   isActive(Round(xyz))        renderer.cu:253 (Round = rintf for float vectors)
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <nanovdb/NanoVDB.h>
#include <nanovdb/util/GridBuilder.h>

using FloatGrid = nanovdb::NanoGrid<float>;
using Vec3fGrid = nanovdb::NanoGrid<nanovdb::Vec3f>;
using FloatLeaf = nanovdb::NanoLeaf<float>;
using Vec3fLeaf = nanovdb::NanoLeaf<nanovdb::Vec3f>;
using CoordT = nanovdb::Coord;
using Vec3fT = nanovdb::Vec3f;

namespace {

struct Dense {
  int reso[3], pad[3];
  const uint8_t* alloc;
  const uint8_t* active;
};

bool allocated(const Dense& d, int i, int j, int k) {
  const int L1 = d.pad[1] / 8, L2 = d.pad[2] / 8;
  return d.alloc[((i >> 3) * L1 + (j >> 3)) * L2 + (k >> 3)] != 0;
}

template <class ValueT>
struct Holder {
  nanovdb::GridHandle<nanovdb::HostBuffer> handle;
  nanovdb::NanoGrid<ValueT>* grid() { return handle.template grid<ValueT>(); }
};

// Every voxel of every allocated leaf gets its value through the build
// accessor (which activates it), then the inactive ones are switched off in
// the NanoVDB leaf masks.
template <class ValueT, class GetV>
Holder<ValueT>* build(const Dense& d, ValueT background, GetV getv) {
  nanovdb::GridBuilder<ValueT> builder(background);
  auto acc = builder.getAccessor();
  for (int i = 0; i < d.pad[0]; ++i)
    for (int j = 0; j < d.pad[1]; ++j)
      for (int k = 0; k < d.pad[2]; ++k)
        if (allocated(d, i, j, k)) acc.setValue(CoordT(i, j, k), getv(i, j, k));
  auto* h = new Holder<ValueT>();
  h->handle = builder.template getHandle<>();
  auto* g = h->grid();
  auto* leaf = g->tree().template getFirstNode<0>();
  const uint32_t nl = g->tree().nodeCount(0);
  for (uint32_t n = 0; n < nl; ++n) {
    for (uint32_t v = 0; v < 512; ++v) {
      const CoordT c = leaf[n].offsetToGlobalCoord(v);
      const int64_t q = (int64_t(c[0]) * d.pad[1] + c[1]) * d.pad[2] + c[2];
      if (!d.active[q]) leaf[n].data()->mValueMask.setOff(v);
    }
  }
  return h;
}

template <class LeafT, class AccT>
typename LeafT::ValueType* leaf_value_ptr(AccT& acc, const CoordT& c) {
  const LeafT* l = acc.template getNode<LeafT>();
  return const_cast<typename LeafT::ValueType*>(&l->data()->mValues[LeafT::CoordToOffset(c)]);
}

}  // namespace

extern "C" {

void* nref_build_float(const int32_t* reso, const int32_t* pad, const uint8_t* alloc,
                       const uint8_t* active, const float* values, float background) {
  Dense d{{reso[0], reso[1], reso[2]}, {pad[0], pad[1], pad[2]}, alloc, active};
  return build<float>(d, background, [&](int i, int j, int k) {
    return values[(int64_t(i) * pad[1] + j) * pad[2] + k];
  });
}

void* nref_build_vec3(const int32_t* reso, const int32_t* pad, const uint8_t* alloc,
                      const uint8_t* active, const float* values, int num, int d3,
                      float background) {
  // values [pad^3, 3*num]; grid d3 takes channels 3*d3 .. 3*d3+2
  Dense d{{reso[0], reso[1], reso[2]}, {pad[0], pad[1], pad[2]}, alloc, active};
  return build<Vec3fT>(d, Vec3fT(background), [&](int i, int j, int k) {
    const float* p = values + ((int64_t(i) * pad[1] + j) * pad[2] + k) * 3 * num + 3 * d3;
    return Vec3fT(p[0], p[1], p[2]);
  });
}

void nref_free_float(void* h) { delete (Holder<float>*)h; }
void nref_free_vec3(void* h) { delete (Holder<Vec3fT>*)h; }

int nref_is_sequential(void* h) { return ((Holder<float>*)h)->grid()->isSequential<0>() ? 1 : 0; }

// ReadAccessor::getValue / isActive (NanoVDB.h:4626-4674)
void nref_lookup_float(void* h, const int32_t* ijk, int64_t n, float* out, uint8_t* act) {
  auto acc = ((Holder<float>*)h)->grid()->getAccessor();
  for (int64_t p = 0; p < n; ++p) {
    const CoordT c(ijk[3 * p], ijk[3 * p + 1], ijk[3 * p + 2]);
    out[p] = acc.getValue(c);
    act[p] = acc.isActive(c) ? 1 : 0;
  }
}

// density_forward_kernel body (densityvdb.cu:110-123)
void nref_density_forward(void* h, const float* xs, const float* ys, const float* zs, int64_t N,
                          float* gpuRes) {
  auto* grid = ((Holder<float>*)h)->grid();
  for (int64_t n = 0; n < N; ++n) {
    auto acc = grid->getAccessor();
    Vec3fT xyz(xs[n], ys[n], zs[n]);
    CoordT ijk = xyz.floor();
    Vec3fT uvw = xyz - ijk.asVec3s();
    gpuRes[n] = 0;
    gpuRes[n] += acc.getValue(ijk) * (1 - uvw[0]) * (1 - uvw[1]) * (1 - uvw[2]); ijk[2] += 1;
    gpuRes[n] += acc.getValue(ijk) * (1 - uvw[0]) * (1 - uvw[1]) * uvw[2]; ijk[1] += 1;
    gpuRes[n] += acc.getValue(ijk) * (1 - uvw[0]) * uvw[1] * uvw[2]; ijk[2] -= 1;
    gpuRes[n] += acc.getValue(ijk) * (1 - uvw[0]) * uvw[1] * (1 - uvw[2]); ijk[0] += 1;
    gpuRes[n] += acc.getValue(ijk) * uvw[0] * uvw[1] * (1 - uvw[2]); ijk[2] += 1;
    gpuRes[n] += acc.getValue(ijk) * uvw[0] * uvw[1] * uvw[2]; ijk[1] -= 1;
    gpuRes[n] += acc.getValue(ijk) * uvw[0] * (1 - uvw[1]) * uvw[2]; ijk[2] -= 1;
    gpuRes[n] += acc.getValue(ijk) * uvw[0] * (1 - uvw[1]) * (1 - uvw[2]);
  }
}

// color_forward_kernel body (colorvdb.cu:16-26, 91-110); grids[d] for d < num
void nref_color_forward(void** hs, int num, const float* xs, const float* ys, const float* zs,
                        int64_t N, float* gpuRes) {
  const int ndim = 3 * num;
  for (int64_t n = 0; n < N; ++n) {
    Vec3fT xyz(xs[n], ys[n], zs[n]);
    CoordT ijk = xyz.floor();
    Vec3fT uvw = xyz - ijk.asVec3s();
    float* p = gpuRes + n * ndim;
    for (int d = 0; d < num; ++d) {
      auto acc = ((Holder<Vec3fT>*)hs[d])->grid()->getAccessor();
      p[0] = 0; p[1] = 0; p[2] = 0;
      auto sv = [&](const CoordT& c, float scale) {
        auto res = acc.getValue(c);
        p[0] += res[0] * scale;
        p[1] += res[1] * scale;
        p[2] += res[2] * scale;
      };
      sv(ijk, (1 - uvw[0]) * (1 - uvw[1]) * (1 - uvw[2])); ijk[2] += 1;
      sv(ijk, (1 - uvw[0]) * (1 - uvw[1]) * uvw[2]); ijk[1] += 1;
      sv(ijk, (1 - uvw[0]) * uvw[1] * uvw[2]); ijk[2] -= 1;
      sv(ijk, (1 - uvw[0]) * uvw[1] * (1 - uvw[2])); ijk[0] += 1;
      sv(ijk, uvw[0] * uvw[1] * (1 - uvw[2])); ijk[2] += 1;
      sv(ijk, uvw[0] * uvw[1] * uvw[2]); ijk[1] -= 1;
      sv(ijk, uvw[0] * (1 - uvw[1]) * uvw[2]); ijk[2] -= 1;
      sv(ijk, uvw[0] * (1 - uvw[1]) * (1 - uvw[2])); ijk[0] -= 1;
      p += 3;
    }
  }
}

// density_backward_kernel body with accumulate (densityvdb.cu:16-27, 152-166):
// the value is added only when the accessor has the corner's leaf cached after
// getValue, i.e. when the corner lies in an allocated leaf.
void nref_density_backward(void* hgrad, const float* xs, const float* ys, const float* zs,
                           const float* grads, int64_t N) {
  auto* grid = ((Holder<float>*)hgrad)->grid();
  for (int64_t n = 0; n < N; ++n) {
    auto acc = grid->getAccessor();
    Vec3fT xyz(xs[n], ys[n], zs[n]);
    CoordT ijk = xyz.floor();
    Vec3fT uvw = xyz - ijk.asVec3s();
    auto accum = [&](const CoordT& c, float val) {
      (void)acc.getValue(c);
      if (acc.isCached<FloatLeaf>(c)) *leaf_value_ptr<FloatLeaf>(acc, c) += val;
    };
    const float g = grads[n];
    accum(ijk, g * (1 - uvw[0]) * (1 - uvw[1]) * (1 - uvw[2])); ijk[2] += 1;
    accum(ijk, g * (1 - uvw[0]) * (1 - uvw[1]) * uvw[2]); ijk[1] += 1;
    accum(ijk, g * (1 - uvw[0]) * uvw[1] * uvw[2]); ijk[2] -= 1;
    accum(ijk, g * (1 - uvw[0]) * uvw[1] * (1 - uvw[2])); ijk[0] += 1;
    accum(ijk, g * uvw[0] * uvw[1] * (1 - uvw[2])); ijk[2] += 1;
    accum(ijk, g * uvw[0] * uvw[1] * uvw[2]); ijk[1] -= 1;
    accum(ijk, g * uvw[0] * (1 - uvw[1]) * uvw[2]); ijk[2] -= 1;
    accum(ijk, g * uvw[0] * (1 - uvw[1]) * (1 - uvw[2]));
  }
}

// color_backward_kernel body (colorvdb.cu:28-37, 141-157), one pass per grid
void nref_color_backward(void** hgrads, int num, const float* xs, const float* ys,
                         const float* zs, const float* grads, int64_t N) {
  const int ndim = 3 * num;
  for (int d = 0; d < num; ++d) {
    auto* grid = ((Holder<Vec3fT>*)hgrads[d])->grid();
    for (int64_t n = 0; n < N; ++n) {
      auto acc = grid->getAccessor();
      const float* src = grads + n * ndim + 3 * d;
      Vec3fT xyz(xs[n], ys[n], zs[n]);
      CoordT ijk = xyz.floor();
      Vec3fT uvw = xyz - ijk.asVec3s();
      auto accum = [&](const CoordT& c, float scale) {
        (void)acc.getValue(c);
        if (acc.isCached<Vec3fLeaf>(c)) {
          Vec3fT* v = leaf_value_ptr<Vec3fLeaf>(acc, c);
          (*v)[0] += src[0] * scale;
          (*v)[1] += src[1] * scale;
          (*v)[2] += src[2] * scale;
        }
      };
      accum(ijk, (1 - uvw[0]) * (1 - uvw[1]) * (1 - uvw[2])); ijk[2] += 1;
      accum(ijk, (1 - uvw[0]) * (1 - uvw[1]) * uvw[2]); ijk[1] += 1;
      accum(ijk, (1 - uvw[0]) * uvw[1] * uvw[2]); ijk[2] -= 1;
      accum(ijk, (1 - uvw[0]) * uvw[1] * (1 - uvw[2])); ijk[0] += 1;
      accum(ijk, uvw[0] * uvw[1] * (1 - uvw[2])); ijk[2] += 1;
      accum(ijk, uvw[0] * uvw[1] * uvw[2]); ijk[1] -= 1;
      accum(ijk, uvw[0] * (1 - uvw[1]) * uvw[2]); ijk[2] -= 1;
      accum(ijk, uvw[0] * (1 - uvw[1]) * (1 - uvw[2]));
    }
  }
}

// Dense read-back [reso^3] (copyToDense semantics through the accessor).
void nref_read_float(void* h, const int32_t* reso, float* out) {
  auto acc = ((Holder<float>*)h)->grid()->getAccessor();
  for (int i = 0; i < reso[0]; ++i)
    for (int j = 0; j < reso[1]; ++j)
      for (int k = 0; k < reso[2]; ++k)
        out[(int64_t(i) * reso[1] + j) * reso[2] + k] = acc.getValue(CoordT(i, j, k));
}

void nref_read_vec3(void** hs, int num, const int32_t* reso, float* out) {
  for (int d = 0; d < num; ++d) {
    auto acc = ((Holder<Vec3fT>*)hs[d])->grid()->getAccessor();
    for (int i = 0; i < reso[0]; ++i)
      for (int j = 0; j < reso[1]; ++j)
        for (int k = 0; k < reso[2]; ++k) {
          const auto v = acc.getValue(CoordT(i, j, k));
          float* p = out + ((int64_t(i) * reso[1] + j) * reso[2] + k) * 3 * num + 3 * d;
          p[0] = v[0]; p[1] = v[1]; p[2] = v[2];
        }
  }
}

// density_updateData / WithPerlr / SkipGrad bodies (densityvdb.cu:197-216,
// 252-273, 309-329) over the sequential leaves.
void nref_density_adam(void* hdata, void* hgrad, void* hm, void* hv, void* hlr, float stepsz,
                       float eps, float beta0, float beta1, int mode) {
  auto* gd = ((Holder<float>*)hdata)->grid();
  auto* gg = ((Holder<float>*)hgrad)->grid();
  auto* gm = ((Holder<float>*)hm)->grid();
  auto* gv = ((Holder<float>*)hv)->grid();
  auto* gl = hlr ? ((Holder<float>*)hlr)->grid() : nullptr;
  const int nleafCount = int(gd->tree().nodeCount(0)) << 9;
  for (int n = 0; n < nleafCount; ++n) {
    const int nleaf = n >> 9, nvox = n & 511;
    auto* leaf_data = gd->tree().getFirstNode<0>() + nleaf;
    if (!leaf_data->isActive(nvox)) continue;
    auto* leaf_grad = gg->tree().getFirstNode<0>() + nleaf;
    auto* leaf_m = gm->tree().getFirstNode<0>() + nleaf;
    auto* leaf_v = gv->tree().getFirstNode<0>() + nleaf;
    const float vgrad = leaf_grad->getValue(nvox);
    if (mode == 1 && vgrad == 0.0f) continue;
    const float vdata = leaf_data->getValue(nvox);
    const float nm = beta0 * leaf_m->getValue(nvox) + (1 - beta0) * vgrad;
    const float nv = beta1 * leaf_v->getValue(nvox) + (1 - beta1) * vgrad * vgrad;
    leaf_m->setValueOnly(nvox, nm);
    leaf_v->setValueOnly(nvox, nv);
    if (mode == 2) {
      const float vperlr = (gl->tree().getFirstNode<0>() + nleaf)->getValue(nvox);
      leaf_data->setValueOnly(nvox, vdata - vperlr * stepsz * nm / (eps + nanovdb::Sqrt(nv)));
    } else {
      leaf_data->setValueOnly(nvox, vdata - stepsz * nm / (eps + nanovdb::Sqrt(nv)));
    }
  }
}

// color_updateData* bodies (colorvdb.cu:193-211, 250-271, 311-330), per grid
void nref_color_adam(void** hdata, void** hgrad, void** hm, void** hv, void* hlr, int num,
                     float stepsz, float eps, float beta0, float beta1, int mode) {
  for (int d = 0; d < num; ++d) {
    auto* gd = ((Holder<Vec3fT>*)hdata[d])->grid();
    auto* gg = ((Holder<Vec3fT>*)hgrad[d])->grid();
    auto* gm = ((Holder<Vec3fT>*)hm[d])->grid();
    auto* gv = ((Holder<Vec3fT>*)hv[d])->grid();
    auto* gl = hlr ? ((Holder<float>*)hlr)->grid() : nullptr;
    const int nleafCount = int(gd->tree().nodeCount(0)) << 9;
    for (int n = 0; n < nleafCount; ++n) {
      const int nleaf = n >> 9, nvox = n & 511;
      auto* leaf_data = gd->tree().getFirstNode<0>() + nleaf;
      if (!leaf_data->isActive(nvox)) continue;
      auto* leaf_grad = gg->tree().getFirstNode<0>() + nleaf;
      auto* leaf_m = gm->tree().getFirstNode<0>() + nleaf;
      auto* leaf_v = gv->tree().getFirstNode<0>() + nleaf;
      const Vec3fT vgrad = leaf_grad->getValue(nvox);
      if (mode == 1 && vgrad == Vec3fT(0.0f)) continue;
      const Vec3fT vdata = leaf_data->getValue(nvox);
      const Vec3fT nm = beta0 * leaf_m->getValue(nvox) + (1 - beta0) * vgrad;
      const Vec3fT nv = beta1 * leaf_v->getValue(nvox) + (1 - beta1) * vgrad * vgrad;
      leaf_m->setValueOnly(nvox, nm);
      leaf_v->setValueOnly(nvox, nv);
      const Vec3fT den(nanovdb::Sqrt(nv[0]) + eps, nanovdb::Sqrt(nv[1]) + eps,
                       nanovdb::Sqrt(nv[2]) + eps);
      const float lrf = mode == 2 ? (gl->tree().getFirstNode<0>() + nleaf)->getValue(nvox) : 1.f;
      Vec3fT upd;
      for (int c = 0; c < 3; ++c)
        upd[c] = mode == 2 ? vdata[c] - lrf * stepsz * nm[c] / den[c]
                           : vdata[c] - stepsz * nm[c] / den[c];
      leaf_data->setValueOnly(nvox, upd);
    }
  }
}

// Index-grid density (renderer.cu:191-220, int() truncation) and the
// isActive(Round(xyz)) test (renderer.cu:253).
void nref_index_density(void* hidx, const float* dendata, const float* xyz, int64_t N, float* out,
                        uint8_t* active_round) {
  auto acc = ((Holder<float>*)hidx)->grid()->getAccessor();
  for (int64_t n = 0; n < N; ++n) {
    Vec3fT p(xyz[3 * n], xyz[3 * n + 1], xyz[3 * n + 2]);
    active_round[n] = acc.isActive(nanovdb::Round<CoordT>(p)) ? 1 : 0;
    int ijk[3] = {int(p[0]), int(p[1]), int(p[2])};
    const float u = p[0] - ijk[0], v = p[1] - ijk[1], w = p[2] - ijk[2];
    CoordT c(ijk[0], ijk[1], ijk[2]);
    int l000 = acc.getValue(c); c[2] += 1;
    int l001 = acc.getValue(c); c[1] += 1;
    int l011 = acc.getValue(c); c[2] -= 1;
    int l010 = acc.getValue(c); c[0] += 1;
    int l110 = acc.getValue(c); c[2] += 1;
    int l111 = acc.getValue(c); c[1] -= 1;
    int l101 = acc.getValue(c); c[2] -= 1;
    int l100 = acc.getValue(c);
    float res = 0;
    res += dendata[l000] * (1 - u) * (1 - v) * (1 - w);
    res += dendata[l001] * (1 - u) * (1 - v) * w;
    res += dendata[l011] * (1 - u) * v * w;
    res += dendata[l010] * (1 - u) * v * (1 - w);
    res += dendata[l110] * u * v * (1 - w);
    res += dendata[l111] * u * v * w;
    res += dendata[l101] * u * (1 - v) * w;
    res += dendata[l100] * u * (1 - v) * (1 - w);
    out[n] = res;
  }
}

}  // extern "C"
