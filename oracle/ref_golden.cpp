/* ref_golden.cpp -- SuperDCA's own solve-path headers behind a C ABI.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by `make -C oracle ref` from the reference
 * sources where they lie (-I <reference>/SuperDCA/include) against the
 * stand-ins in oracle/ref_shims, into oracle/_ref/libref_plmdca.so.  It is
 * used in this container to pin the C oracle and to write the golden fixtures
 * under tests/golden; nothing on the GPU side loads it.
 *
 * Reference code exercised (file:line within the SuperDCA project):
 *   plmDCA_objective_fval_and_gradient      include/plmDCA_objective.hpp:38-249
 *   plmDCA_optimizer_parameters (lambda rule, r-state cache, views)
 *                                           include/plmDCA_optimizer_parameters.hpp:100-373
 *   calculate_weights                       include/plmDCA_optimizer_parameters.hpp:39-98
 *   Coupling_matrix_view(+accumulator)      include/Coupling_matrix_view.hpp:30-212
 *   ising_gauge / frobenius_norm            include/plmDCA_utility.hpp:57-83,
 *                                           include/Matrix_math.hpp:166-213
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <limits>
#include <memory>
#include <numeric>
#include <vector>

#include "apegrunt/Alignment.h"

namespace superdca {
/* Stand-in for the static option getters the parameter class reads
 * (SuperDCA/include/plmDCA_options.h). */
struct plmDCA_options {
    static double s_threshold, s_lambda_h, s_lambda_J;
    static double reweighting_threshold() { return s_threshold; }
    static bool verbose() { return false; }
    static std::ostream *out_stream() { return &std::cout; }
    static double lambda_h() { return s_lambda_h; }
    static double lambda_J() { return s_lambda_J; }
    static void set_lambda_h(double v) { s_lambda_h = v; }
    static void set_lambda_J(double v) { s_lambda_J = v; }
};
double plmDCA_options::s_threshold = 0.9;
double plmDCA_options::s_lambda_h = -1.0;
double plmDCA_options::s_lambda_J = -1.0;
} // namespace superdca

#include "plmDCA_objective.hpp"
#include "plmDCA_utility.hpp"

using state_t = apegrunt::triallelic_state_t;
using params_t = superdca::plmDCA_optimizer_parameters<double, state_t>;

namespace {
struct RefProblem {
    std::vector<apegrunt::Alignment_ptr<state_t>> alignments;
    std::shared_ptr<std::vector<double>> weights;
    std::unique_ptr<params_t> params;
    std::size_t D = 0;
};

template <typename T> T *aligned_copy(const T *src, std::size_t n)
{
    void *p = nullptr;
    if (posix_memalign(&p, 64, sizeof(T) * n + 64) != 0) return nullptr;
    if (src) std::memcpy(p, src, sizeof(T) * n);
    else std::memset(p, 0, sizeof(T) * n);
    return static_cast<T *>(p);
}
} // namespace

extern "C" {

/* weights: NULL selects the reference's calculate_weights at `threshold`. */
void *ref_problem_new(const uint8_t *states, int64_t N, int64_t L, const double *weights,
                      double threshold, double lambda_h_opt, double lambda_J_opt)
{
    auto *p = new RefProblem;
    p->alignments.push_back(std::make_shared<apegrunt::Alignment<state_t>>(states, N, L, nullptr));
    superdca::plmDCA_options::s_threshold = threshold;
    superdca::plmDCA_options::s_lambda_h = lambda_h_opt;
    superdca::plmDCA_options::s_lambda_J = lambda_J_opt;
    if (weights)
        p->weights = std::make_shared<std::vector<double>>(weights, weights + N);
    else
        p->weights = std::make_shared<std::vector<double>>(
            superdca::calculate_weights<state_t, double>(p->alignments.back()));
    p->params.reset(new params_t(p->alignments, p->weights));
    p->D = p->params->get_dimensions();
    return p;
}

void ref_problem_free(void *h) { delete static_cast<RefProblem *>(h); }

int64_t ref_dim(void *h) { return int64_t(static_cast<RefProblem *>(h)->D); }

void ref_lambdas(void *h, double *lambda_h, double *lambda_J)
{
    auto *p = static_cast<RefProblem *>(h);
    *lambda_h = p->params->get_lambda_h();
    *lambda_J = p->params->get_lambda_J();
}

void ref_weights(void *h, double *w)
{
    auto *p = static_cast<RefProblem *>(h);
    std::copy(p->weights->begin(), p->weights->end(), w);
}

double ref_objective(void *h, int64_t r, const double *x, double *g)
{
    auto *p = static_cast<RefProblem *>(h);
    double *xa = aligned_copy(x, p->D);
    double *ga = aligned_copy<double>(nullptr, p->D);
    p->params->set_target_column(std::size_t(r));
    p->params->set_solution(xa);
    p->params->set_gradient(ga, true);
    superdca::plmDCA_objective_fval_and_gradient<params_t, double>(*p->params);
    const double f = p->params->get_fvalue();
    if (g) std::memcpy(g, ga, sizeof(double) * p->D);
    std::free(xa);
    std::free(ga);
    return f;
}

/* Score row of a solved locus as include/plmDCA.hpp:378-393 computes it. */
void ref_score_row(void *h, int64_t r, const double *x, int64_t gap, float *row)
{
    auto *p = static_cast<RefProblem *>(h);
    double *xa = aligned_copy(x, p->D);
    auto &&Jr = p->params->get_Jr_view(xa);
    const std::size_t L = Jr.size();
    for (std::size_t n = 0; n < L; ++n) {
        if (int64_t(n) == r) {
            row[n] = std::numeric_limits<float>::quiet_NaN();
            continue;
        }
        float v;
        if (int64_t(n) < r)
            v = superdca::frobenius_norm(superdca::ising_gauge(Jr, n, true), std::size_t(gap));
        else
            v = superdca::frobenius_norm(superdca::ising_gauge(Jr, n), std::size_t(gap));
        row[n] = v;
    }
    std::free(xa);
}

} // extern "C"
