// A Chombo-side caller of the C ABI, compiled from C++ by the test suite.
//
// The bodies of LinElastPatchGodunov::updateState / plasticUpdate and of
// LinElastLevelGodunov::define / step below are the ones a maintainer puts
// into the reference's classes (srcLinElast/LinElastPatchGodunov.H:63-83,
// srcLinElast/LinElastPatchGodunov.cpp:101-129, srcLinElast/LinElastPhysics.cpp:544-554,
// srcLinElast/LinElastLevelGodunov.H:91-114, srcLinElast/LinElastLevelGodunov.cpp:45-167,174-398).
// Box, FArrayBox, FluxBox, ProblemDomain and MayDay are minimal stand-ins for
// Chombo's classes with the members those bodies touch: FABs alias caller
// memory (Chombo's FArrayBox(const Box&, int, Real*) alias constructor), and
// MayDay::Error throws so that the test entry points can return the status.
//
// Built with g++ -std=c++17 -Wall -Wextra -Werror -pedantic against
// include/tetemoko_gb300.h and linked to libtetemoko_gb300.so; the extern "C"
// functions at the end are what the tests call through ctypes.
#include "tetemoko_gb300.h"

#include <stdexcept>
#include <string>
#include <vector>

typedef double Real;

// ------------------------------------------------------------ stand-ins
class IntVect {
 public:
  IntVect(int i = 0, int j = 0) : m_v{i, j} {}
  int operator[](int d) const { return m_v[d]; }

 private:
  int m_v[2];
};

class Box {
 public:
  Box() : m_lo(0, 0), m_hi(-1, -1) {}
  Box(const IntVect& lo, const IntVect& hi) : m_lo(lo), m_hi(hi) {}
  int smallEnd(int d) const { return m_lo[d]; }
  int bigEnd(int d) const { return m_hi[d]; }
  // the face box of direction `dir` (Chombo's surroundingNodes)
  Box surroundingNodes(int dir) const {
    return Box(m_lo, IntVect(m_hi[0] + (dir == 0 ? 1 : 0), m_hi[1] + (dir == 1 ? 1 : 0)));
  }
  bool operator==(const Box& o) const {
    return m_lo[0] == o.m_lo[0] && m_lo[1] == o.m_lo[1] && m_hi[0] == o.m_hi[0] && m_hi[1] == o.m_hi[1];
  }

 private:
  IntVect m_lo, m_hi;
};

class FArrayBox {
 public:
  FArrayBox() : m_ncomp(0), m_data(nullptr) {}
  FArrayBox(const Box& b, int ncomp, Real* alias) : m_box(b), m_ncomp(ncomp), m_data(alias) {}
  const Box& box() const { return m_box; }
  int nComp() const { return m_ncomp; }
  Real* dataPtr() { return m_data; }
  const Real* dataPtr() const { return m_data; }

 private:
  Box m_box;
  int m_ncomp;
  Real* m_data;
};

struct ShimError : std::runtime_error {
  tmk_status status;
  ShimError(const std::string& what, tmk_status st) : std::runtime_error(what), status(st) {}
};

namespace MayDay {
[[noreturn]] void Error(const char* msg, tmk_status st) { throw ShimError(msg, st); }
}  // namespace MayDay

// Chombo's FluxBox allocates its face FABs in resize(); here they alias the
// caller's arrays and resize() checks that they cover the faces of the box.
class FluxBox {
 public:
  FluxBox(FArrayBox* fx, FArrayBox* fy) : m_f{fx, fy} {}
  void resize(const Box& b, int ncomp) {
    for (int d = 0; d < 2; ++d)
      if (!m_f[d] || !(m_f[d]->box() == b.surroundingNodes(d)) || m_f[d]->nComp() != ncomp)
        MayDay::Error("FluxBox::resize: face FAB does not cover the faces of the box", TMK_ERR_BAD_DESC);
  }
  FArrayBox& operator[](int d) { return *m_f[d]; }
  bool defined() const { return m_f[0] && m_f[1]; }

 private:
  FArrayBox* m_f[2];
};

class ProblemDomain {
 public:
  explicit ProblemDomain(const Box& b = Box()) : m_box(b) {}
  const Box& domainBox() const { return m_box; }

 private:
  Box m_box;
};

// the library context and stream a Chombo build keeps beside its physics object
static tmk_context* s_ctx = nullptr;
static void* s_stream = nullptr;

static tmk_box toBox(const Box& b) {
  tmk_box t = {{b.smallEnd(0), b.smallEnd(1)}, {b.bigEnd(0), b.bigEnd(1)}};
  return t;
}

static tmk_fab toFab(FArrayBox& f) {
  tmk_fab t = {f.dataPtr(), {f.box().smallEnd(0), f.box().smallEnd(1)},
               {f.box().bigEnd(0), f.box().bigEnd(1)}, f.nComp()};
  return t;
}

// ------------------------------------------------------------ patch level
class LinElastPatchGodunov {
 public:
  LinElastPatchGodunov(const ProblemDomain& domain, Real dx)
      : m_domain(domain), m_dx(dx), m_currentTime(0.0), m_bdryData(nullptr) {}
  void setCurrentTime(const Real& t) { m_currentTime = t; }
  void setCurrentBox(const Box& b) { m_currentBox = b; }
  // LEPhysIBC::setBdryData: a non-owning pointer to the patch's fault FAB
  void setBdryData(FArrayBox* B) { m_bdryData = B; }

  void updateState(FArrayBox& a_U, FluxBox& a_F, Real& a_maxWaveSpeed, const FArrayBox& a_S, const Real& a_dt,
                   const Box& a_box) {
    (void)a_S;                                       // the reference's source term is unused
    tmk_fab U = toFab(a_U);
    tmk_fab Fx, Fy, *pFx = nullptr, *pFy = nullptr;
    if (a_F.defined()) {
      a_F.resize(a_box, a_U.nComp());
      Fx = toFab(a_F[0]);
      Fy = toFab(a_F[1]);
      pFx = &Fx;
      pFy = &Fy;
    }
    tmk_fab Bf, *B = nullptr;
    if (m_bdryData) {
      Bf = toFab(*m_bdryData);
      B = &Bf;
    }
    const tmk_box valid = toBox(a_box);
    const tmk_box dom = toBox(m_domain.domainBox());
    const tmk_status st = tmk_patch_update_state(s_ctx, &U, B, pFx, pFy, &valid, &dom, m_dx, m_currentTime, a_dt,
                                                 &a_maxWaveSpeed, s_stream);
    if (st != TMK_OK) MayDay::Error("tmk_patch_update_state failed", st);
  }

  // LinElastPhysics::plasticUpdate
  void plasticUpdate(FArrayBox& a_U, const Box& a_box, const Real& a_dt) {
    tmk_fab U = toFab(a_U);
    const tmk_box b = toBox(a_box);
    const tmk_status st = tmk_plastic_update(s_ctx, &U, &b, a_dt, s_stream);
    if (st != TMK_OK) MayDay::Error("tmk_plastic_update failed", st);
  }

 private:
  ProblemDomain m_domain;
  Real m_dx;
  Real m_currentTime;
  Box m_currentBox;
  FArrayBox* m_bdryData;
};

// ------------------------------------------------------------ level
class LinElastLevelGodunov {
 public:
  LinElastLevelGodunov() : m_tmkLevel(nullptr), m_hasCoarser(false) {}
  ~LinElastLevelGodunov() { tmk_level_destroy(m_tmkLevel); }

  void define(const std::vector<Box>& a_grids, const ProblemDomain& a_domain, Real a_dx) {
    std::vector<tmk_box> boxes;
    for (const Box& b : a_grids) boxes.push_back(toBox(b));
    const tmk_box dom = toBox(a_domain.domainBox());
    tmk_level_destroy(m_tmkLevel);
    m_tmkLevel = nullptr;
    const tmk_status st = tmk_level_create(s_ctx, &dom, a_dx, (int)boxes.size(), boxes.data(), &m_tmkLevel);
    if (st != TMK_OK) MayDay::Error("tmk_level_create failed", st);
  }

  void setPatch(int p, const Real* U, const Real* B, int host) {
    const tmk_status st = tmk_level_set_patch(m_tmkLevel, p, U, B, host);
    if (st != TMK_OK) MayDay::Error("tmk_level_set_patch failed", st);
  }

  void getPatch(int p, Real* U, Real* B, int host) {
    const tmk_status st = tmk_level_get_patch(m_tmkLevel, p, U, B, host);
    if (st != TMK_OK) MayDay::Error("tmk_level_get_patch failed", st);
  }

  // LinElastLevelGodunov::step for a level without a coarser level; the
  // state, fault data and flux registers are the device-resident copies
  Real step(const Real& a_TCoarseOld, const Real& a_TCoarseNew, const Real& a_time, const Real& a_dt) {
    double dtNew = 0.0;
    tmk_status st;
    if (m_hasCoarser)
      st = tmk_level_step_cf(m_tmkLevel, a_time, a_dt, a_TCoarseOld, a_TCoarseNew, s_stream, &dtNew);
    else
      st = tmk_level_step(m_tmkLevel, a_time, a_dt, s_stream, &dtNew);
    if (st != TMK_OK) MayDay::Error("LinElastLevelGodunov::step failed", st);
    return dtNew;
  }

 private:
  tmk_level* m_tmkLevel;
  bool m_hasCoarser;
};

static LinElastLevelGodunov* s_level = nullptr;

// ------------------------------------------------------------ test entry points
namespace {
Box boxOf(const int* lohi) { return Box(IntVect(lohi[0], lohi[1]), IntVect(lohi[2], lohi[3])); }

template <class F>
int guarded(F&& f) {
  try {
    f();
  } catch (const ShimError& e) {
    return (int)e.status;
  }
  return (int)TMK_OK;
}
}  // namespace

extern "C" {

int shim_context_create(const tmk_elastic_params* e, const tmk_scheme* s, const tmk_rs_params* rs,
                        const tmk_sw_params* sw, const tmk_plastic_params* pl) {
  return guarded([&] {
    tmk_context_destroy(s_ctx);
    s_ctx = nullptr;
    const tmk_status st = tmk_context_create(e, s, rs, sw, pl, &s_ctx);
    if (st != TMK_OK) MayDay::Error("tmk_context_create failed", st);
  });
}

void shim_context_destroy(void) {
  tmk_context_destroy(s_ctx);
  s_ctx = nullptr;
}

// ubox, bbox, valid, domain: (lo0, lo1, hi0, hi1); B, Fx, Fy may be NULL
int shim_patch_update_state(double* U, const int* ubox, double* B, const int* bbox, int nb, double* Fx, double* Fy,
                            const int* valid, const int* domain, double dx, double time, double dt, double* mws) {
  return guarded([&] {
    const Box vb = boxOf(valid);
    FArrayBox Uf(boxOf(ubox), TMK_NCOMP, U);
    FArrayBox Bf = B ? FArrayBox(boxOf(bbox), nb, B) : FArrayBox();
    FArrayBox Fxf(vb.surroundingNodes(0), TMK_NCOMP, Fx), Fyf(vb.surroundingNodes(1), TMK_NCOMP, Fy);
    FluxBox F(Fx ? &Fxf : nullptr, Fy ? &Fyf : nullptr);
    FArrayBox S;
    LinElastPatchGodunov pg(ProblemDomain(boxOf(domain)), dx);
    pg.setCurrentTime(time);
    pg.setCurrentBox(vb);
    pg.setBdryData(B ? &Bf : nullptr);
    Real maxWaveSpeed = 0.0;
    pg.updateState(Uf, F, maxWaveSpeed, S, dt, vb);
    *mws = maxWaveSpeed;
  });
}

int shim_plastic_update(double* U, const int* ubox, const int* box, const int* domain, double dx, double dt) {
  return guarded([&] {
    FArrayBox Uf(boxOf(ubox), TMK_NCOMP, U);
    LinElastPatchGodunov pg(ProblemDomain(boxOf(domain)), dx);
    pg.plasticUpdate(Uf, boxOf(box), dt);
  });
}

// boxes: n x (lo0, lo1, hi0, hi1)
int shim_level_define(const int* domain, double dx, int n, const int* boxes) {
  return guarded([&] {
    std::vector<Box> grids;
    for (int p = 0; p < n; ++p) grids.push_back(boxOf(boxes + 4 * p));
    if (!s_level) s_level = new LinElastLevelGodunov();
    s_level->define(grids, ProblemDomain(boxOf(domain)), dx);
  });
}

int shim_level_set_patch(int p, const double* U, const double* B, int host) {
  return guarded([&] {
    if (!s_level) MayDay::Error("no level", TMK_ERR_BAD_DESC);
    s_level->setPatch(p, U, B, host);
  });
}

int shim_level_get_patch(int p, double* U, double* B, int host) {
  return guarded([&] {
    if (!s_level) MayDay::Error("no level", TMK_ERR_BAD_DESC);
    s_level->getPatch(p, U, B, host);
  });
}

int shim_level_step(double time, double dt, double* dt_new) {
  return guarded([&] {
    if (!s_level) MayDay::Error("no level", TMK_ERR_BAD_DESC);
    *dt_new = s_level->step(0.0, 0.0, time, dt);
  });
}

void shim_level_destroy(void) {
  delete s_level;
  s_level = nullptr;
}

}  // extern "C"
