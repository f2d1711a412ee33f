// extern "C" shim over the reference's own operator classes, compiled from
// the reference sources where they lie (see oracle/build_ref.sh).  Test
// infrastructure only: it lets the tests and the golden-fixture script run the
// unmodified reference perform_op / orbit tables / moments on the CPU.
//
// Dispatch mirrors TMat/pfunc.cpp:16-106 (model, dim, axialdir -> operator),
// with extend_cond passed through exactly as pfunc passes `multieigs`
// (TMat/pfunc.cpp:22) so callers can select the reference driver semantics.
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "tmat.hpp"
#include "tmat3d.hpp"
#include "tmatreduce.hpp"

namespace {

struct RefOp {
  virtual ~RefOp() {}
  virtual int64_t rows() const = 0;
  virtual double normfactor() const = 0;
  virtual void perform(const double* x, double* y) const = 0;
  virtual int has_transpose() const { return 0; }
  virtual void perform_t(const double* x, double* y) const { perform(x, y); }
  virtual int64_t orbit(uint64_t* idx, uint32_t* dup, int64_t cap) const { return -1; }
  virtual int moments(const double* ql, const double* qr, double* out) const { return -1; }
  virtual int phys(const double* ql, const double* qr, double* out, int cap) const { return -1; }
};

template <class Op>
struct SymBase : RefOp {
  std::unique_ptr<Op> op;
  int layer;
  explicit SymBase(Op* p, int lsize) : op(p), layer(lsize) {}
  int64_t rows() const override { return (int64_t)op->rows(); }
  double normfactor() const override { return op->getnormfactor(); }
  void perform(const double* x, double* y) const override { op->perform_op(x, y); }
  int moments(const double* ql, const double* qr, double* out) const override {
    return op->moments(layer, ql, qr, out);
  }
  int phys(const double* ql, const double* qr, double* out, int cap) const override {
    std::vector<double> r;
    int st = op->phys_extend(layer, ql, qr, r);
    int n = (int)r.size();
    for (int i = 0; i < n && i < cap; ++i) out[i] = r[i];
    return st < 0 ? -1 - n : n;
  }
};

template <class Op>
struct SymReduced : SymBase<Op> {
  using SymBase<Op>::SymBase;
  int64_t orbit(uint64_t* idx, uint32_t* dup, int64_t cap) const override {
    int64_t n = this->rows();
    for (int64_t i = 0; i < n && i < cap; ++i) {
      auto pr = this->op->getIrrepState((SPIN_TYPE)i);
      idx[i] = pr.first;
      dup[i] = pr.second;
    }
    return n;
  }
};

template <class Op>
struct GenPhys : RefOp {
  int layer;
  explicit GenPhys(int lsize) : layer(lsize) {}
  virtual const Op& get() const = 0;
  int moments(const double* ql, const double* qr, double* out) const override {
    int64_t n = rows();
    std::vector<std::complex<double> > cl(ql, ql + n), cr(qr, qr + n);
    return get().moments(layer, cl.data(), cr.data(), out);
  }
  int phys(const double* ql, const double* qr, double* out, int cap) const override {
    int64_t n = rows();
    std::vector<std::complex<double> > cl(ql, ql + n), cr(qr, qr + n);
    std::vector<double> r;
    int st = get().phys_extend(layer, cl.data(), cr.data(), r);
    int m = (int)r.size();
    for (int i = 0; i < m && i < cap; ++i) out[i] = r[i];
    return st < 0 ? -1 - m : m;
  }
};

// general operator whose transpose holds a reference to the parent
template <class Op, class OpT>
struct GenRefT : GenPhys<Op> {
  std::unique_ptr<Op> op;
  std::unique_ptr<OpT> opt;
  GenRefT(Op* p, int lsize) : GenPhys<Op>(lsize), op(p), opt(new OpT(*p)) {}
  const Op& get() const override { return *op; }
  int64_t rows() const override { return (int64_t)op->rows(); }
  double normfactor() const override { return op->getnormfactor(); }
  void perform(const double* x, double* y) const override { op->perform_op(x, y); }
  int has_transpose() const override { return 1; }
  void perform_t(const double* x, double* y) const override { opt->perform_op(x, y); }
};

template <class Op, class OpT>
struct GenReducedT : GenRefT<Op, OpT> {
  using GenRefT<Op, OpT>::GenRefT;
  int64_t orbit(uint64_t* idx, uint32_t* dup, int64_t cap) const override {
    int64_t n = this->rows();
    for (int64_t i = 0; i < n && i < cap; ++i) {
      auto pr = this->op->getIrrepState((SPIN_TYPE)i);
      idx[i] = pr.first;
      dup[i] = pr.second;
    }
    return n;
  }
};

// YAT: the transpose is an independent instance built from the parameters
struct YATHolder : GenPhys<TMat::YATMatVecProd2D> {
  std::unique_ptr<TMat::YATMatVecProd2D> op;
  std::unique_ptr<TMat::YATMatVecProd2D_T> opt;
  YATHolder(const MParameter& mp)
      : GenPhys<TMat::YATMatVecProd2D>(mp.size), op(new TMat::YATMatVecProd2D(mp)),
        opt(new TMat::YATMatVecProd2D_T(mp)) {}
  const TMat::YATMatVecProd2D& get() const override { return *op; }
  int64_t rows() const override { return (int64_t)op->rows(); }
  double normfactor() const override { return op->getnormfactor(); }
  void perform(const double* x, double* y) const override { op->perform_op(x, y); }
  int has_transpose() const override { return 1; }
  void perform_t(const double* x, double* y) const override { opt->perform_op(x, y); }
};

struct Y2ATHolder : GenPhys<TMat::Y2ATMatVecProd2D> {
  std::unique_ptr<TMat::Y2ATMatVecProd2D> op;
  explicit Y2ATHolder(const MParameter& mp)
      : GenPhys<TMat::Y2ATMatVecProd2D>(mp.size), op(new TMat::Y2ATMatVecProd2D(mp)) {}
  const TMat::Y2ATMatVecProd2D& get() const override { return *op; }
  int64_t rows() const override { return (int64_t)op->rows(); }
  double normfactor() const override { return op->getnormfactor(); }
  void perform(const double* x, double* y) const override { op->perform_op(x, y); }
};

}  // namespace

extern "C" {

void* ref_create(char model, int dim, int axialdir, int extend_cond, double betaJ, double kappa,
                 double kappa2, double h, int size) {
  MParameter mp;
  mp.betaJ = betaJ;
  mp.kappa = kappa;
  mp.kappa2 = kappa2;
  mp.h = h;
  mp.size = size;
  const int ec = extend_cond;
  int lsize = size;
  if (dim == 3) lsize = (size >> 16) * (size & 0xffff);
  using namespace TMat;
  if (model == 'A' && dim == 2) {
    switch (axialdir) {
      case 0: return new Y2ATHolder(mp);
      case 1: return new SymBase<XATMatVecProd2D>(new XATMatVecProd2D(mp), lsize);
      case 2: return new YATHolder(mp);
      case 5: return new SymReduced<XAMMatVecProd2D>(new XAMMatVecProd2D(mp, ec), lsize);
      case 6:
        return new GenReducedT<YAMMatVecProd2D, YAMMatVecProd2D_T>(new YAMMatVecProd2D(mp, ec), lsize);
      case 9: return new SymBase<XATMatVecProd2D>(new XATMatVecProd2D(mp, 1), lsize);
      case 13: return new SymReduced<XAMMatVecProd2D>(new XAMMatVecProd2D(mp, ec | 1), lsize);
      case 17: case 18:
        return new SymBase<XATMatVecProd2D>(new XATMatVecProd2D(mp, (axialdir & 1) ? 5 : 9), lsize);
      case 19: case 20:
        return new SymBase<XATMatVecProd2D>(new XATMatVecProd2D(mp, (axialdir & 1) ? 13 : 17), lsize);
      default: return nullptr;
    }
  }
  if (model == 'A' && dim == 3) {
    if (axialdir == 1) return new SymReduced<XAMMatVecProd3D>(new XAMMatVecProd3D(mp, ec), lsize);
    return nullptr;
  }
  if (model == 'B') {
    switch (axialdir) {
      case 3:
        return new GenRefT<ZBTMatVecProd2D, ZBTMatVecProd2D_T>(new ZBTMatVecProd2D(mp), lsize);
      case 6:
        return new GenReducedT<YAMMatVecProd2D, YAMMatVecProd2D_T>(new YBMMatVecProd2D(mp, ec), lsize);
      case 7:
        return new GenReducedT<ZBMMatVecProd2D, ZBMMatVecProd2D_T>(new ZBMMatVecProd2D(mp, ec), lsize);
      default: return nullptr;
    }
  }
  if (model == 'D') {
    switch (axialdir) {
      case 1: case 2: return new SymBase<XDTMatVecProd2D>(new XDTMatVecProd2D(mp), lsize);
      case 5: case 6: return new SymReduced<XDMMatVecProd2D>(new XDMMatVecProd2D(mp, ec), lsize);
      case 17: case 18:
        return new SymBase<XDTMatVecProd2D>(new XDTMatVecProd2D(mp, (axialdir & 1) ? 5 : 9), lsize);
      default: return nullptr;
    }
  }
  return nullptr;
}

void ref_destroy(void* p) { delete static_cast<RefOp*>(p); }
int64_t ref_rows(void* p) { return static_cast<RefOp*>(p)->rows(); }
double ref_normfactor(void* p) { return static_cast<RefOp*>(p)->normfactor(); }
void ref_perform_op(void* p, const double* x, double* y) { static_cast<RefOp*>(p)->perform(x, y); }
int ref_has_transpose(void* p) { return static_cast<RefOp*>(p)->has_transpose(); }
void ref_perform_op_t(void* p, const double* x, double* y) { static_cast<RefOp*>(p)->perform_t(x, y); }
int64_t ref_orbit(void* p, uint64_t* idx, uint32_t* dup, int64_t cap) {
  return static_cast<RefOp*>(p)->orbit(idx, dup, cap);
}
int ref_moments(void* p, const double* ql, const double* qr, double* out4) {
  return static_cast<RefOp*>(p)->moments(ql, qr, out4);
}
int ref_phys_extend(void* p, const double* ql, const double* qr, double* out, int cap) {
  return static_cast<RefOp*>(p)->phys(ql, qr, out, cap);
}
int ref_opcount(void) { return OpCounter::get(); }

}  // extern "C"
