// Level-A drop-in: the reference's CUDA plugin point implemented on the GB300 engine.
//
// The reference compiles src/cuda_box.cu into its solver library when SOVEREIGN_CUDA is defined
// (02-software/solver/CMakeLists.txt:6-14); solve_accelerated_box then calls
//     std::unique_ptr<BoxIteration> make_cuda_box(const CsrMatrix&, cost, lower, upper, lipschitz)
//     std::string cuda_device_name()
// (include/accelerated_qp.hpp:9-16).  This translation unit provides exactly those two symbols
// over the C-ABI of libboxqp.so (bqp_box_*): build the reference library with this file in place
// of src/cuda_box.cu, define SOVEREIGN_CUDA=1, and link libboxqp.so.  The reference's own loop,
// CLI (--backend cuda) and scale harness then iterate on the GB300 kernels; each step() is one
// fused FISTA iteration with the CPU loop's rounding (division by L, no FMA contraction), so the
// CUDA backend reproduces the CPU backend's iterates.
//
// Errors follow src/cuda_box.cu:7,35: std::runtime_error("CUDA: ...") and
// "No CUDA device available".
#include "accelerated_qp.hpp"
#include "boxqp.h"

#include <stdexcept>
#include <string>
#include <vector>

namespace sovereign {
namespace {

class GB300Box : public BoxIteration {
public:
    GB300Box(const CsrMatrix& h, const std::vector<double>& c, const std::vector<double>& lo,
             const std::vector<double>& up, double lipschitz)
        : n_(static_cast<int64_t>(c.size())) {
        box_ = bqp_box_create(0, n_, static_cast<int64_t>(h.value.size()), h.start.data(), h.index.data(),
                              h.value.data(), c.data(), lo.data(), up.data(), lipschitz);
        if (!box_) {
            std::string why = bqp_box_last_error(nullptr);
            if (why == "No CUDA device available") throw std::runtime_error(why);
            throw std::runtime_error("CUDA: " + why);
        }
    }
    ~GB300Box() override { bqp_box_destroy(box_); }
    GB300Box(const GB300Box&) = delete;
    GB300Box& operator=(const GB300Box&) = delete;

    void step(double momentum) override {
        if (bqp_box_step(box_, momentum) != BQP_OK) throw std::runtime_error(bqp_box_last_error(box_));
    }
    std::vector<double> primal() override {
        std::vector<double> x(static_cast<size_t>(n_));
        if (bqp_box_primal(box_, x.data()) != BQP_OK) throw std::runtime_error(bqp_box_last_error(box_));
        return x;
    }

private:
    int64_t n_;
    bqp_box* box_ = nullptr;
};

}  // namespace

std::unique_ptr<BoxIteration> make_cuda_box(const CsrMatrix& h, const std::vector<double>& cost,
                                            const std::vector<double>& lower, const std::vector<double>& upper,
                                            double lipschitz) {
    return std::unique_ptr<BoxIteration>(new GB300Box(h, cost, lower, upper, lipschitz));
}

std::string cuda_device_name() {
    char name[256];
    if (bqp_device_name(0, name, sizeof(name)) != BQP_OK) return "No CUDA device available";
    return name;
}

}  // namespace sovereign
