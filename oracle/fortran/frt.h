// frt.h - run-time support of the Fortran-subset translator (test
// infrastructure).
//
// The translator turns the reference's Fortran 90 into C++ that includes
// this header.  It supplies:
//   * Arr<T>: a Fortran array (any lower bounds, column-major, strided views)
//     whose element addresses follow Fortran's address arithmetic;
//   * the intrinsic functions the reference calls;
//   * a one-rank MPI: every call the reference makes with a single process
//     (sends to itself are buffered by tag and delivered at the matching
//     receive or wait; reductions copy);
//   * the FFTW 2 Fortran interface for the plans the reference creates
//     (1D complex transforms and 1D in-place real transforms, unnormalised,
//     sign -1 forward), evaluated as direct sums with exactly reduced
//     twiddle angles.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace frt {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

using cplx = std::complex<double>;

struct Bound {
  int64_t lo, hi;
};

template <class T>
struct Arr {
  T* p = nullptr;           // address of the element at the lower bounds
  int rank = 0;
  int64_t lb[7] = {0}, ub[7] = {0}, st[7] = {0};
  std::shared_ptr<std::vector<T>> own;
  T* abase = nullptr;       // allocation range (0 for views of unknown extent)
  size_t an = 0;

  Arr() = default;
  explicit Arr(std::initializer_list<Bound> b) { allocate(b); }

  bool allocated() const { return p != nullptr; }

  void allocate(std::initializer_list<Bound> b) {
    rank = (int)b.size();
    int64_t n = 1;
    int d = 0;
    for (const Bound& x : b) {
      lb[d] = x.lo;
      ub[d] = x.hi;
      st[d] = n;
      const int64_t e = x.hi - x.lo + 1;
      n *= e > 0 ? e : 0;
      ++d;
    }
    own = std::make_shared<std::vector<T>>((size_t)n, T());
    p = own->data();
    abase = p;
    an = (size_t)n;
  }
  void deallocate() {
    own.reset();
    p = nullptr;
    abase = nullptr;
    an = 0;
  }

  // view of caller memory with the callee's declared bounds (explicit-shape
  // dummy argument, sequence association)
  static Arr view(T* ptr, std::initializer_list<Bound> b) {
    Arr a;
    a.rank = (int)b.size();
    int64_t n = 1;
    int d = 0;
    for (const Bound& x : b) {
      a.lb[d] = x.lo;
      a.ub[d] = x.hi;
      a.st[d] = n;
      const int64_t e = x.hi - x.lo + 1;
      n *= e > 0 ? e : 0;
      ++d;
    }
    a.p = ptr;
    return a;
  }

  int64_t lbound(int d) const { return lb[d - 1]; }
  int64_t ubound(int d) const { return ub[d - 1]; }
  int64_t extent(int d) const {
    const int64_t e = ub[d - 1] - lb[d - 1] + 1;
    return e > 0 ? e : 0;
  }
  int64_t size() const {
    int64_t n = 1;
    for (int d = 1; d <= rank; ++d) n *= extent(d);
    return n;
  }
  T* data() const { return p; }

  T& at(int64_t off) const {
    T* q = p + off;
    if (abase && (q < abase || q >= abase + an))
      throw Error("array reference outside the allocation");
    return *q;
  }
  T& operator()(int64_t i0) const { return at((i0 - lb[0]) * st[0]); }
  T& operator()(int64_t i0, int64_t i1) const {
    return at((i0 - lb[0]) * st[0] + (i1 - lb[1]) * st[1]);
  }
  T& operator()(int64_t i0, int64_t i1, int64_t i2) const {
    return at((i0 - lb[0]) * st[0] + (i1 - lb[1]) * st[1] + (i2 - lb[2]) * st[2]);
  }
  T& operator()(int64_t i0, int64_t i1, int64_t i2, int64_t i3) const {
    return at((i0 - lb[0]) * st[0] + (i1 - lb[1]) * st[1] + (i2 - lb[2]) * st[2] +
              (i3 - lb[3]) * st[3]);
  }
  T& operator()(int64_t i0, int64_t i1, int64_t i2, int64_t i3, int64_t i4) const {
    return at((i0 - lb[0]) * st[0] + (i1 - lb[1]) * st[1] + (i2 - lb[2]) * st[2] +
              (i3 - lb[3]) * st[3] + (i4 - lb[4]) * st[4]);
  }
};

// ---- intrinsics ------------------------------------------------------------
inline double dble(double x) { return x; }
inline int32_t fint(double x) { return (int32_t)x; }            // truncation
inline int32_t nint(double x) { return (int32_t)std::lround(x); }  // half away from 0
inline int32_t imod(int32_t a, int32_t b) { return a % b; }
inline int64_t imod(int64_t a, int64_t b) { return a % b; }
inline double rmod(double a, double b) { return std::fmod(a, b); }
inline double sign(double a, double b) { return b >= 0.0 ? std::fabs(a) : -std::fabs(a); }
inline int32_t sign(int32_t a, int32_t b) { return b >= 0 ? std::abs(a) : -std::abs(a); }
template <class A, class B>
inline auto fmax2(A a, B b) -> decltype(a + b) { return a > b ? a : b; }
template <class A, class B>
inline auto fmin2(A a, B b) -> decltype(a + b) { return a < b ? a : b; }
template <class A>
inline A fmaxn(A a) { return a; }
template <class A>
inline A fminn(A a) { return a; }
template <class A, class B, class... R>
inline auto fmaxn(A a, B b, R... r) { return fmaxn(fmax2(a, b), r...); }
template <class A, class B, class... R>
inline auto fminn(A a, B b, R... r) { return fminn(fmin2(a, b), r...); }
inline int32_t ipow(int32_t b, int32_t e) {
  int32_t r = 1;
  for (int32_t i = 0; i < e; ++i) r *= b;
  return r;
}
// x**n for integer n as repeated multiplication from the left
inline double rpowi(double x, int32_t n) {
  if (n == 0) return 1.0;
  if (n < 0) return 1.0 / rpowi(x, -n);
  double r = x;
  for (int32_t i = 1; i < n; ++i) r = r * x;
  return r;
}
inline std::string trim(const std::string& s) {
  size_t e = s.find_last_not_of(' ');
  return e == std::string::npos ? std::string() : s.substr(0, e + 1);
}
inline int64_t cshift_index(int64_t t, int64_t shift, int64_t ext) {
  int64_t r = (t + shift) % ext;
  return r < 0 ? r + ext : r;
}

[[noreturn]] inline void stop(const char* where) {
  throw Error(std::string("STOP at ") + where);
}

// ---- one-rank MPI ------------------------------------------------------------
namespace mpi {
enum { COMM_WORLD = 91, REAL8 = 1, INTEGER = 2, DOUBLE_PRECISION = 3, LOGICAL = 4,
       REAL = 5, COMPLEX16 = 6, DOUBLE_COMPLEX = 7, SUM = 11, MAX = 12, MIN = 13,
       STATUS_SIZE = 6, ANY_SOURCE = -1, PROD = 14 };

inline size_t type_size(int t) {
  switch (t) {
    case REAL8: case DOUBLE_PRECISION: case REAL: return 8;  // default real is 8 bytes
    case INTEGER: case LOGICAL: return 4;
    case COMPLEX16: case DOUBLE_COMPLEX: return 16;
  }
  throw Error("MPI: unknown datatype");
}

struct Message {
  int tag;
  std::vector<char> data;
};
struct PendingRecv {
  void* buf;
  size_t bytes;
  int tag;
  bool done;
};
struct World {
  std::deque<Message> queue;
  std::vector<PendingRecv> recvs;  // request handles index into this
};
inline World& world() {
  static World w;
  return w;
}
inline void deliver_pending() {
  World& w = world();
  for (PendingRecv& r : w.recvs) {
    if (r.done) continue;
    for (auto it = w.queue.begin(); it != w.queue.end(); ++it) {
      if (it->tag == r.tag) {
        if (it->data.size() != r.bytes) throw Error("MPI: message size mismatch");
        std::memcpy(r.buf, it->data.data(), r.bytes);
        w.queue.erase(it);
        r.done = true;
        break;
      }
    }
  }
}
}  // namespace mpi

inline void mpi_init(int32_t& ierr) { ierr = 0; }
inline void mpi_finalize(int32_t& ierr) { ierr = 0; }
inline void mpi_comm_rank(int32_t, int32_t& rank, int32_t& ierr) { rank = 0; ierr = 0; }
inline void mpi_comm_size(int32_t, int32_t& n, int32_t& ierr) { n = 1; ierr = 0; }
inline void mpi_barrier(int32_t, int32_t& ierr) { ierr = 0; }
inline double mpi_wtime() { return 0.0; }
inline void mpi_bcast(void*, int32_t, int32_t, int32_t, int32_t, int32_t& ierr) { ierr = 0; }
inline void mpi_allreduce(void* s, void* r, int32_t n, int32_t t, int32_t, int32_t,
                          int32_t& ierr) {
  if (s != r) std::memmove(r, s, (size_t)n * mpi::type_size(t));
  ierr = 0;
}
inline void mpi_reduce(void* s, void* r, int32_t n, int32_t t, int32_t, int32_t, int32_t,
                       int32_t& ierr) {
  if (s != r) std::memmove(r, s, (size_t)n * mpi::type_size(t));
  ierr = 0;
}
inline void mpi_isend(void* buf, int32_t n, int32_t t, int32_t dest, int32_t tag, int32_t,
                      int32_t& req, int32_t& ierr) {
  if (dest != 0) throw Error("MPI: send to a rank other than 0");
  mpi::Message m;
  m.tag = tag;
  m.data.resize((size_t)n * mpi::type_size(t));
  if (n) std::memcpy(m.data.data(), buf, m.data.size());
  mpi::world().queue.push_back(std::move(m));
  req = -1;  // a buffered send is complete at once
  ierr = 0;
}
inline void mpi_send(void* buf, int32_t n, int32_t t, int32_t dest, int32_t tag, int32_t,
                     int32_t& ierr) {
  int32_t req;
  mpi_isend(buf, n, t, dest, tag, 0, req, ierr);
}
inline void mpi_irecv(void* buf, int32_t n, int32_t t, int32_t src, int32_t tag, int32_t,
                      int32_t& req, int32_t& ierr) {
  if (src != 0 && src != mpi::ANY_SOURCE) throw Error("MPI: receive from a rank other than 0");
  mpi::World& w = mpi::world();
  w.recvs.push_back({buf, (size_t)n * mpi::type_size(t), tag, false});
  req = (int32_t)w.recvs.size() - 1;
  ierr = 0;
}
inline void mpi_wait_one(int32_t req) {
  if (req < 0) return;
  mpi::deliver_pending();
  mpi::World& w = mpi::world();
  if (req >= (int32_t)w.recvs.size() || !w.recvs[req].done)
    throw Error("MPI: receive without a matching send (deadlock)");
}
inline void mpi_waitall(int32_t n, int32_t* reqs, void*, int32_t& ierr) {
  mpi::deliver_pending();
  for (int32_t i = 0; i < n; ++i) mpi_wait_one(reqs[i]);
  bool all = true;
  for (auto& r : mpi::world().recvs) all = all && r.done;
  if (all) mpi::world().recvs.clear();
  ierr = 0;
}
inline void mpi_wait(int32_t& req, void*, int32_t& ierr) {
  mpi_wait_one(req);
  ierr = 0;
}
inline void mpi_recv(void* buf, int32_t n, int32_t t, int32_t src, int32_t tag, int32_t,
                     void*, int32_t& ierr) {
  int32_t req;
  mpi_irecv(buf, n, t, src, tag, 0, req, ierr);
  mpi_wait_one(req);
}
inline void mpi_sendrecv(void* sb, int32_t sn, int32_t st, int32_t dest, int32_t stag,
                         void* rb, int32_t rn, int32_t rt, int32_t src, int32_t rtag, int32_t,
                         void*, int32_t& ierr) {
  mpi_send(sb, sn, st, dest, stag, 0, ierr);
  mpi_recv(rb, rn, rt, src, rtag, 0, nullptr, ierr);
}

// ---- FFTW 2 Fortran interface ------------------------------------------------
struct Plan {
  int n;
  int sign;       // -1 forward, +1 backward
  bool real;      // rfftwnd (real <-> complex) plan
};
inline std::vector<Plan>& plans() {
  static std::vector<Plan> p;
  return p;
}
// e^{sign 2 pi i jk / n} with jk reduced mod n first (exact argument reduction)
inline cplx twiddle(int64_t jk, int n, int sign) {
  const int64_t r = jk % n;
  const double a = 2.0 * M_PI * (double)r / (double)n;
  return cplx(std::cos(a), sign * std::sin(a));
}
inline void fftw_f77_create_plan_(int64_t& plan, int32_t n, int32_t dir, int32_t) {
  plans().push_back({n, dir, false});
  plan = (int64_t)plans().size() - 1;
}
inline void rfftwnd_f77_create_plan_(int64_t& plan, int32_t rank, int32_t n, int32_t dir,
                                     int32_t) {
  if (rank != 1) throw Error("rfftwnd plan of rank > 1 is not emulated");
  plans().push_back({n, dir, true});
  plan = (int64_t)plans().size() - 1;
}
inline void fftw_f77_destroy_plan_(int64_t&) {}
inline void rfftwnd_f77_destroy_plan_(int64_t&) {}
// out-of-place complex DFT of length n
inline void fftw_f77_one_(int64_t& plan, cplx* in, cplx* out) {
  const Plan& P = plans().at((size_t)plan);
  std::vector<cplx> r((size_t)P.n);
  for (int k = 0; k < P.n; ++k) {
    cplx s(0.0, 0.0);
    for (int j = 0; j < P.n; ++j) s += in[j] * twiddle((int64_t)j * k, P.n, P.sign);
    r[(size_t)k] = s;
  }
  for (int k = 0; k < P.n; ++k) out[k] = r[(size_t)k];
}
// in place, real <-> n/2+1 complex values interleaved in n+2 reals
inline void rfftwnd_f77_one_real_to_complex_(int64_t& plan, double* v, int32_t) {
  const Plan& P = plans().at((size_t)plan);
  const int n = P.n;
  std::vector<double> x(v, v + n);
  for (int k = 0; k <= n / 2; ++k) {
    cplx s(0.0, 0.0);
    for (int j = 0; j < n; ++j) s += x[(size_t)j] * twiddle((int64_t)j * k, n, -1);
    v[2 * k] = s.real();
    v[2 * k + 1] = s.imag();
  }
}
inline void rfftwnd_f77_one_complex_to_real_(int64_t& plan, double* v, int32_t) {
  const Plan& P = plans().at((size_t)plan);
  const int n = P.n;
  std::vector<cplx> c((size_t)(n / 2 + 1));
  for (int k = 0; k <= n / 2; ++k) c[(size_t)k] = cplx(v[2 * k], v[2 * k + 1]);
  for (int j = 0; j < n; ++j) {
    // Hermitian extension: c(n-k) = conj(c(k))
    double s = 0.0;
    for (int k = 0; k < n; ++k) {
      cplx ck = k <= n / 2 ? c[(size_t)k] : std::conj(c[(size_t)(n - k)]);
      if (k == 0 || (n % 2 == 0 && k == n / 2)) ck = cplx(ck.real(), 0.0);
      s += (ck * twiddle((int64_t)j * k, n, +1)).real();
    }
    v[j] = s;
  }
}

// IFPORT's generator is not published: a translated program that draws from
// it cannot be reproduced, so it fails loudly.
inline void srand(int32_t) { throw Error("IFPORT srand/rand are not reproducible"); }
inline double rand() { throw Error("IFPORT srand/rand are not reproducible"); }
inline int32_t irand() { throw Error("IFPORT srand/rand are not reproducible"); }

// parameter overrides (name -> value) applied when a module is initialised
inline std::map<std::string, double>& overrides() {
  static std::map<std::string, double> m;
  return m;
}
template <class T>
inline T param(const char* name, T dflt) {
  auto it = overrides().find(name);
  return it == overrides().end() ? dflt : (T)it->second;
}

}  // namespace frt
