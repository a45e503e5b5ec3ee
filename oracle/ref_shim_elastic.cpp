/*
 * ref_shim_elastic.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiles the reference's own elastic source-injection and receiver CPU code
 * (included by include path from the reference checkout; nothing is copied
 * into this repository) and exposes it with C linkage:
 *   deps/CustomOps/SourceOps/AddSource.cpp   (forwardCPU / backwardCPU)
 *   deps/CustomOps/ReceiveOps/GetReceive.cpp (forward / backward)
 */
#include <cstdint>
#include "AddSource.cpp"
#include "GetReceive.cpp"

extern "C" {

void ref_add_source_fwd(double* out5, const double* in5, int64_t nsrc, const int64_t* srci,
                        const int64_t* srcj, const int64_t* srctype, const double* srcv,
                        int64_t NX, int64_t NY) {
  const int64_t N = (NX + 2) * (NY + 2);
  /* forwardCPU's outputs are (vx_, vy_, sigmaxx_, sigmayy_, sigmaxy_) */
  forwardCPU(out5, out5 + N, out5 + 2 * N, out5 + 3 * N, out5 + 4 * N, in5, in5 + N,
             in5 + 2 * N, in5 + 3 * N, in5 + 4 * N, (const int64*)srci, (const int64*)srcj,
             srcv, (const int64*)srctype, nsrc, NX, NY);
}

void ref_add_source_bwd(double* gin5, double* grad_srcv, const double* gout5, int64_t nsrc,
                        const int64_t* srci, const int64_t* srcj, const int64_t* srctype,
                        int64_t NX, int64_t NY) {
  const int64_t N = (NX + 2) * (NY + 2);
  backwardCPU(gin5, gin5 + N, gin5 + 2 * N, gin5 + 3 * N, gin5 + 4 * N, grad_srcv, gout5,
              gout5 + N, gout5 + 2 * N, gout5 + 3 * N, gout5 + 4 * N, (const int64*)srci,
              (const int64*)srcj, nullptr, (const int64*)srctype, nsrc, NX, NY);
}

void ref_get_receive_fwd(double* out, const double* vx, const double* vy,
                         const double* sxx, const double* syy, const double* sxy,
                         int64_t nt, int64_t nrcv, const int64_t* rcvi, const int64_t* rcvj,
                         const int64_t* rcvtype, int64_t NX, int64_t NY) {
  forward(out, vx, vy, sxx, syy, sxy, nt, (const int64*)rcvi, (const int64*)rcvj,
          (const int64*)rcvtype, nrcv, NX, NY);
}

void ref_get_receive_bwd(double* gvx, double* gvy, double* gsxx, double* gsyy,
                         double* gsxy, const double* gout, int64_t nt, int64_t nrcv,
                         const int64_t* rcvi, const int64_t* rcvj, const int64_t* rcvtype,
                         int64_t NX, int64_t NY) {
  backward(gvx, gvy, gsxx, gsyy, gsxy, gout, nt, (const int64*)rcvi, (const int64*)rcvj,
           (const int64*)rcvtype, nrcv, NX, NY);
}

}  // extern "C"
