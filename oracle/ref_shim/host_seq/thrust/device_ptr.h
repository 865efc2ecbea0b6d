// Sequential host stand-in (writer-pin build only): the reference's
// report_force (output.cu:22-49) sums two arrays with thrust::reduce over
// thrust::device_ptr.  In the host build the "device" arrays are host memory;
// the reduction runs left to right (thrust's device reduction order is its
// own, so sums agree to rounding).
#pragma once
#include <cstddef>

namespace thrust {
template <class T>
struct device_ptr {
    T *p;
    explicit device_ptr(T *q) : p(q) {}
    device_ptr operator+(std::ptrdiff_t n) const { return device_ptr(p + n); }
};
template <class T, class Op>
T reduce(device_ptr<T> first, device_ptr<T> last, T init, Op op) {
    for (T *q = first.p; q != last.p; ++q) init = op(init, *q);
    return init;
}
}  // namespace thrust
