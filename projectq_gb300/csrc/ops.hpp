// Plain host types shared by the planners and the kernel launchers (no CUDA
// headers, so the planners also build in host-only test harnesses).
#pragma once

#include <complex>
#include <cstdint>
#include <vector>

namespace gsim {

using cplx = std::complex<double>;

// One controlled dense k-qubit gate on bit positions pos[] (matrix bit l is
// pos[l]); the gate acts where (index & ctrl_mask) == ctrl_mask.
struct DenseOp {
  std::vector<cplx> m;        // 2^k x 2^k, row-major, FP64
  std::vector<unsigned> pos;  // k distinct bit positions
  uint64_t ctrl_mask = 0;
};

}  // namespace gsim
