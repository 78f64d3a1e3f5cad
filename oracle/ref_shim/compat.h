/* Forward-compatibility shim for compiling the reference's Thrust host code
 * with the CUDA 13 Thrust headers and the CPP (host) device system.  It only
 * re-adds what newer Thrust removed and the reference still names:
 * the adaptable-function bases (functors.h:8, gen_mod_pep.cu:160), the
 * binary_traits used by its vendored bind1st/bind2nd (functional.hpp:33-37),
 * and headers that older Thrust included transitively (sort.cu:33). */
#pragma once
#include <cuda_runtime.h>
#include <thrust/functional.h>
#include <thrust/sequence.h>
namespace thrust {
template <typename A, typename R> struct unary_function { typedef A argument_type; typedef R result_type; };
template <typename A, typename B, typename R> struct binary_function {
    typedef A first_argument_type; typedef B second_argument_type; typedef R result_type; };
template <typename Op> struct binary_traits;
template <template <class> class F, typename T> struct binary_traits<F<T>> {
    typedef F<T> function_type;
    typedef const F<T> &param_type;
    typedef T first_argument_type;
    typedef T second_argument_type;
    typedef T result_type;
};
}
