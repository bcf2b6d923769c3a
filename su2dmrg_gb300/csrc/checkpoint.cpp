// Checkpoint files of the engine, read and written from device buffers:
//   * an MPS tensor per site, uu-<ns>-<D>-<S>-<ky>-<exc>-<pos>.{dat,bin}
//     (dmrg_su2::save_mps2 / read_mps, dmrg_su2_omp.cpp:864-1067): the .dat
//     holds the structure as text ("nbond<TAB>locspin", then per leg
//     "dir<TAB>n", the n values of 2j each followed by a TAB, the n multiplet
//     counts likewise), the .bin one int presence flag per block, the reduced
//     blocks back to back (tensor_su2::get_telement, tensor_su2.cpp:566-581:
//     exactly the packed layout of this library) and then each stored
//     block's Clebsch-Gordan tensor in the same order;
//   * the energies, enr-<ns>-<D>-<S>-<ky>-<exc>.dat (save_enr / read_enr,
//     :1070-1151): one value per line with 16 significant digits, appended;
//   * the bond weights, ww-<ns>-<D>-<S>-<ky>-<exc>-<ns/2>.bin (save_ww /
//     read_ww, :1154-1242): raw doubles.
// The engine keeps canonical CG parts (make_cgc for 3-leg tensors), so they
// are written from the sector labels; on reading, each block's CG part is
// checked to be proportional to the canonical one and the reduced block is
// rescaled by the ratio (1 for files the engine wrote).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "kernels.hpp"
#include "su2_meta.hpp"
#include "su2g.h"

namespace {

int fail(int code, const std::string& msg) { return su2g::set_last_error(code, msg); }

struct File {
  FILE* f = nullptr;
  File(const char* path, const char* mode) { f = path ? std::fopen(path, mode) : nullptr; }
  ~File() {
    if (f) std::fclose(f);
  }
  File(const File&) = delete;
  File& operator=(const File&) = delete;
};

// Canonical CG part of block b: make_cgc for 3 legs; for 2 legs the identity
// of a scalar operator (directions +1, -1) or the singlet of a vector.
bool canonical_cg(const su2g::Struct& s, int b, std::vector<double>* out) {
  if (s.nbond == 3) {
    const int a0 = s.block_angm(b, 0), a1 = s.block_angm(b, 1), a2 = s.block_angm(b, 2);
    out->assign((size_t)(a0 + 1) * (a1 + 1) * (a2 + 1), 0.0);
    su2g::make_cgc(a0, a1, a2, out->data());
    return true;
  }
  if (s.nbond == 2) {
    const int a = s.block_angm(b, 0);
    out->assign((size_t)(a + 1) * (a + 1), 0.0);
    if (s.legs[0].dir == 1 && s.legs[1].dir == -1) {
      for (int i = 0; i <= a; ++i) (*out)[(size_t)i * (a + 1) + i] = 1.0;
    } else {
      su2g::make_singlet(a, out->data());
    }
    return true;
  }
  return false;
}

int64_t block_size(const su2g::Struct& s, int b) {
  int64_t n = 1;
  for (int l = 0; l < s.nbond; ++l) n *= s.block_dim(b, l);
  return n;
}

// .dat -> desc; false with *err on a malformed file
bool read_dat(const char* path, std::vector<int>* desc, std::string* err) {
  File f(path, "r");
  if (!f.f) {
    *err = std::string("cannot open ") + (path ? path : "(null)");
    return false;
  }
  int nb = 0, lc = 0;
  if (std::fscanf(f.f, "%d %d", &nb, &lc) != 2 || nb < 1 || nb > su2g::kMaxLegs) {
    *err = "malformed structure header";
    return false;
  }
  desc->assign({nb, lc});
  for (int l = 0; l < nb; ++l) {
    int dir = 0, n = 0;
    if (std::fscanf(f.f, "%d %d", &dir, &n) != 2 || n < 1 || n > 4096) {
      *err = "malformed leg header";
      return false;
    }
    desc->push_back(dir);
    desc->push_back(n);
    for (int k = 0; k < 2 * n; ++k) {
      int v = 0;
      if (std::fscanf(f.f, "%d", &v) != 1) {
        *err = "truncated leg";
        return false;
      }
      desc->push_back(v);
    }
  }
  return true;
}

// Parsed checkpoint of one tensor: structure, flags, reduced data (rescaled to
// the canonical CG), on the host.
int load_host(const char* dat, const char* bin, su2g::Struct* s, std::vector<int>* desc, std::vector<double>* data) {
  std::string e;
  if (!read_dat(dat, desc, &e)) return fail(SU2G_EIO, "mps_load: " + e);
  if (!s->parse(desc->data(), &e)) return fail(SU2G_EIO, "mps_load: structure: " + e);
  File f(bin, "rb");
  if (!f.f) return fail(SU2G_EIO, std::string("mps_load: cannot open ") + (bin ? bin : "(null)"));
  std::vector<int> flag(s->nten);
  if (std::fread(flag.data(), sizeof(int), flag.size(), f.f) != flag.size())
    return fail(SU2G_EIO, "mps_load: truncated flags");
  for (int& v : flag) v = v ? 1 : 0;
  s->set_layout(flag.data());
  int64_t n2 = 0;
  std::vector<std::vector<double>> cg(s->nten);
  for (int b = 0; b < s->nten; ++b) {
    if (!s->flag[b]) continue;
    if (!canonical_cg(*s, b, &cg[b])) return fail(SU2G_EUNSUPPORTED, "mps_load: tensors of 1 or more than 3 legs");
    n2 += (int64_t)cg[b].size();
  }
  data->assign(std::max<int64_t>(s->total, 1), 0.0);
  std::vector<double> cgf(std::max<int64_t>(n2, 1));
  if (std::fread(data->data(), sizeof(double), s->total, f.f) != (size_t)s->total ||
      std::fread(cgf.data(), sizeof(double), n2, f.f) != (size_t)n2)
    return fail(SU2G_EIO, "mps_load: truncated data");
  if (std::fgetc(f.f) != EOF) return fail(SU2G_EIO, "mps_load: trailing bytes after the CG part");
  // each block's CG part against the canonical one: rescale by the ratio
  int64_t p = 0;
  for (int b = 0; b < s->nten; ++b) {
    if (!s->flag[b]) continue;
    const std::vector<double>& c0 = cg[b];
    const double* c1 = cgf.data() + p;
    p += (int64_t)c0.size();
    size_t k = 0;
    for (size_t i = 1; i < c0.size(); ++i)
      if (std::fabs(c0[i]) > std::fabs(c0[k])) k = i;
    const double lam = c1[k] / c0[k];
    bool same = true, prop = lam != 0.0 && std::isfinite(lam);
    for (size_t i = 0; i < c0.size() && prop; ++i) {
      if (c1[i] != c0[i]) same = false;
      if (std::fabs(c1[i] - lam * c0[i]) > 1e-12 * std::fabs(lam * c0[k])) prop = false;
    }
    if (same) continue;
    if (!prop) return fail(SU2G_EUNSUPPORTED, "mps_load: a block's CG part is not proportional to the canonical one");
    double* x = data->data() + s->offset[b];
    const int64_t n = block_size(*s, b);
    for (int64_t i = 0; i < n; ++i) x[i] *= lam;
  }
  return SU2G_OK;
}

}  // namespace

extern "C" int su2g_checkpoint_name(int kind, int ns, int dcut, int totspin, int ky, int exc, int pos, char* buf,
                                    int cap) {
  if (!buf || cap <= 0) return fail(SU2G_EINVAL, "checkpoint_name: no buffer");
  int n;
  switch (kind) {
    case SU2G_CKPT_MPS_DAT: n = std::snprintf(buf, cap, "uu-%d-%d-%d-%d-%d-%d.dat", ns, dcut, totspin, ky, exc, pos); break;
    case SU2G_CKPT_MPS_BIN: n = std::snprintf(buf, cap, "uu-%d-%d-%d-%d-%d-%d.bin", ns, dcut, totspin, ky, exc, pos); break;
    case SU2G_CKPT_ENR: n = std::snprintf(buf, cap, "enr-%d-%d-%d-%d-%d.dat", ns, dcut, totspin, ky, exc); break;
    case SU2G_CKPT_WW: n = std::snprintf(buf, cap, "ww-%d-%d-%d-%d-%d-%d.bin", ns, dcut, totspin, ky, exc, pos); break;
    default: return fail(SU2G_EINVAL, "checkpoint_name: unknown kind");
  }
  if (n < 0 || n >= cap) return fail(SU2G_EINVAL, "checkpoint_name: buffer too small");
  return SU2G_OK;
}

extern "C" int su2g_mps_save(const char* dat_path, const char* bin_path, su2g_tensor t, void* stream) {
  su2g::Struct s;
  std::string e;
  if (!t.desc || !s.parse(t.desc, &e)) return fail(SU2G_EINVAL, "mps_save: " + e);
  s.set_layout(t.flag);
  if (s.total > 0 && !t.data) return fail(SU2G_EINVAL, "mps_save: null data");
  std::vector<double> cg;
  std::vector<std::vector<double>> cgs(s.nten);
  for (int b = 0; b < s.nten; ++b)
    if (s.flag[b] && !canonical_cg(s, b, &cgs[b]))
      return fail(SU2G_EUNSUPPORTED, "mps_save: tensors of 1 or more than 3 legs");
  std::vector<double> host(std::max<int64_t>(s.total, 1));
  if (s.total > 0) {
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t ce = cudaMemcpyAsync(host.data(), t.data, s.total * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return fail(SU2G_ECUDA, std::string("mps_save: ") + cudaGetErrorString(ce));
  }
  {
    File f(dat_path, "w");
    if (!f.f) return fail(SU2G_EIO, std::string("mps_save: cannot create ") + (dat_path ? dat_path : "(null)"));
    std::fprintf(f.f, "%d\t%d\n", s.nbond, s.locspin);
    for (int l = 0; l < s.nbond; ++l) {
      std::fprintf(f.f, "%d\t%d\n", s.legs[l].dir, s.legs[l].n());
      for (int a : s.legs[l].angm) std::fprintf(f.f, "%d\t", a);
      std::fprintf(f.f, "\n");
      for (int d : s.legs[l].dim) std::fprintf(f.f, "%d\t", d);
      std::fprintf(f.f, "\n");
    }
    if (std::ferror(f.f)) return fail(SU2G_EIO, "mps_save: write error (.dat)");
  }
  File f(bin_path, "wb");
  if (!f.f) return fail(SU2G_EIO, std::string("mps_save: cannot create ") + (bin_path ? bin_path : "(null)"));
  std::vector<int> flag(s.flag.begin(), s.flag.end());
  bool ok = std::fwrite(flag.data(), sizeof(int), flag.size(), f.f) == flag.size();
  ok = ok && std::fwrite(host.data(), sizeof(double), s.total, f.f) == (size_t)s.total;
  for (int b = 0; b < s.nten && ok; ++b)
    if (s.flag[b]) ok = std::fwrite(cgs[b].data(), sizeof(double), cgs[b].size(), f.f) == cgs[b].size();
  if (!ok) return fail(SU2G_EIO, "mps_save: write error (.bin)");
  return SU2G_OK;
}

extern "C" int su2g_mps_load_layout(const char* dat_path, const char* bin_path, int* out_desc, int out_desc_cap,
                                    int* out_flag, int out_flag_cap, int64_t* out_len) {
  su2g::Struct s;
  std::vector<int> desc;
  std::vector<double> data;
  int rc = load_host(dat_path, bin_path, &s, &desc, &data);
  if (rc) return rc;
  if (!out_desc || !out_flag || (int)desc.size() > out_desc_cap || s.nten > out_flag_cap)
    return fail(SU2G_EINVAL, "mps_load_layout: output arrays too small");
  std::copy(desc.begin(), desc.end(), out_desc);
  std::copy(s.flag.begin(), s.flag.end(), out_flag);
  if (out_len) *out_len = s.total;
  return SU2G_OK;
}

extern "C" int su2g_mps_load(const char* dat_path, const char* bin_path, double* out, int64_t out_cap, void* stream) {
  su2g::Struct s;
  std::vector<int> desc;
  std::vector<double> data;
  int rc = load_host(dat_path, bin_path, &s, &desc, &data);
  if (rc) return rc;
  if (s.total > out_cap || (s.total > 0 && !out)) return fail(SU2G_EINVAL, "mps_load: output buffer too small");
  if (s.total == 0) return SU2G_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t ce = cudaMemcpyAsync(out, data.data(), s.total * sizeof(double), cudaMemcpyHostToDevice, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) return fail(SU2G_ECUDA, std::string("mps_load: ") + cudaGetErrorString(ce));
  return SU2G_OK;
}

extern "C" int su2g_enr_append(const char* path, double value) {
  File f(path, "a");
  if (!f.f) return fail(SU2G_EIO, std::string("enr_append: cannot open ") + (path ? path : "(null)"));
  if (std::fprintf(f.f, "%.16g\n", value) < 0) return fail(SU2G_EIO, "enr_append: write error");
  return SU2G_OK;
}

extern "C" int su2g_enr_read(const char* path, double* values, int cap, int* count) {
  File f(path, "r");
  if (!f.f) return fail(SU2G_EIO, std::string("enr_read: cannot open ") + (path ? path : "(null)"));
  int n = 0;
  double v;
  while (std::fscanf(f.f, "%lf", &v) == 1) {
    if (values && n < cap) values[n] = v;
    ++n;
  }
  if (count) *count = n;
  if (n > cap) return fail(SU2G_EINVAL, "enr_read: more values than cap (" + std::to_string(n) + ")");
  return SU2G_OK;
}

extern "C" int su2g_ww_save(const char* path, const double* ww, int64_t n) {
  if (n < 0 || (n > 0 && !ww)) return fail(SU2G_EINVAL, "ww_save: bad arguments");
  File f(path, "wb");
  if (!f.f) return fail(SU2G_EIO, std::string("ww_save: cannot create ") + (path ? path : "(null)"));
  if (std::fwrite(ww, sizeof(double), n, f.f) != (size_t)n) return fail(SU2G_EIO, "ww_save: write error");
  return SU2G_OK;
}

extern "C" int su2g_ww_load(const char* path, double* ww, int64_t n, int64_t* nread) {
  if (n < 0 || (n > 0 && !ww)) return fail(SU2G_EINVAL, "ww_load: bad arguments");
  File f(path, "rb");
  if (!f.f) return fail(SU2G_EIO, std::string("ww_load: cannot open ") + (path ? path : "(null)"));
  const size_t got = std::fread(ww, sizeof(double), n, f.f);
  if (nread) *nread = (int64_t)got;
  return SU2G_OK;
}
