// extern "C" forwarders onto the reference's C++ entry points (include/core.h:9-19), so
// that Python tests can call the reference core.cpp built in oracle/_ref by plain names.
// Test infrastructure only.
#include <cstddef>
#include <cstdint>
double base_gauss_lower(int, double*, uint64_t*, int*, double*, double*);
double base_gauss_upper(int, double*, uint64_t*, int*, double*, double*, int);
double base_gauss_upper_new(int, double*, uint64_t*, int*, double*, double*, int);
double supernodal_upper(size_t, int*, double*, double*, int*, uint64_t*, int, int);
double supernodal_upper_new(size_t, int*, double*, double*, int*, uint64_t*, int, int);
double supernodal_blas_upper(int, int, size_t, int*, double*, double*, uint64_t*, int*, int);
double ccs2ccs_pad(double*, int*, uint64_t*, double*, uint64_t*, int*, int*, int&, int&);
int setLevelUpAndGetMaxLevel(int, int*, uint64_t*, uint64_t*);
double barrier_upper(int, double*, double*, double*, int*, uint64_t*, int, int);
double barrier_upper_new(int, double*, double*, double*, int*, uint64_t*, int, int);

extern "C" {
double ref_base_gauss_lower(int n, double* v, uint64_t* r, int* c, double* x, double* b) { return base_gauss_lower(n, v, r, c, x, b); }
double ref_base_gauss_upper(int n, double* v, uint64_t* r, int* c, double* x, double* b, int rhs) { return base_gauss_upper(n, v, r, c, x, b, rhs); }
double ref_base_gauss_upper_new(int n, double* v, uint64_t* r, int* c, double* x, double* b, int rhs) { return base_gauss_upper_new(n, v, r, c, x, b, rhs); }
double ref_supernodal_upper(size_t sn, int* s, double* x, double* v, int* c, uint64_t* r, int n, int rhs) { return supernodal_upper(sn, s, x, v, c, r, n, rhs); }
double ref_supernodal_upper_new(size_t sn, int* s, double* x, double* v, int* c, uint64_t* r, int n, int rhs) { return supernodal_upper_new(sn, s, x, v, c, r, n, rhs); }
double ref_supernodal_blas_upper(int n, int nz, size_t sn, int* s, double* x, double* v, uint64_t* ci, int* rp, int rhs) { return supernodal_blas_upper(n, nz, sn, s, x, v, ci, rp, rhs); }
int ref_ccs2ccs_pad(double* v, int* c, uint64_t* r, double* vp, uint64_t* cp, int* rp, int* nodes, int sn) { int s = sn, nz = 0; ccs2ccs_pad(v, c, r, vp, cp, rp, nodes, s, nz); return nz; }
int ref_set_levels(int n, int* c, uint64_t* r, uint64_t* lv) { return setLevelUpAndGetMaxLevel(n, c, r, lv); }
double ref_barrier_upper(int n, double* x, double* b, double* v, int* c, uint64_t* r, int nt, int rhs) { return barrier_upper(n, x, b, v, c, r, nt, rhs); }
double ref_barrier_upper_new(int n, double* x, double* b, double* v, int* c, uint64_t* r, int nt, int rhs) { return barrier_upper_new(n, x, b, v, c, r, nt, rhs); }
}
