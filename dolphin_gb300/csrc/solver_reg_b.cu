// Register-solver instances for K = 18 .. 32 slots (K slots, G threads per pixel
// group); the instances are spread over several translation units so that they compile
// in parallel.
#include "dpl_common.cuh"
#include "pix_args.cuh"
#include "solver.cuh"
#include "solver_reg.cuh"

namespace dpl {

dpl_status launch_solve_reg_b(int K, int G, const PixArgs& a, cudaStream_t s) {
    if (K == 18 && G == 32) return launch_solve_reg_k<18, 32>(a, s);
    if (K == 20 && G == 32) return launch_solve_reg_k<20, 32>(a, s);
    if (K == 22 && G == 32) return launch_solve_reg_k<22, 32>(a, s);
    if (K == 24 && G == 32) return launch_solve_reg_k<24, 32>(a, s);
    if (K == 26 && G == 32) return launch_solve_reg_k<26, 32>(a, s);
    if (K == 28 && G == 32) return launch_solve_reg_k<28, 32>(a, s);
    if (K == 30 && G == 32) return launch_solve_reg_k<30, 32>(a, s);
    if (K == 32 && G == 32) return launch_solve_reg_k<32, 32>(a, s);
    return fail(DPL_ERR_UNSUPPORTED, "register solver: no instance for this slot count and group size");
}

}  // namespace dpl
