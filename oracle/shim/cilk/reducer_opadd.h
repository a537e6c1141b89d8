/* Minimal stand-in for <cilk/reducer_opadd.h>: an atomic accumulator with the
 * two operations the reference uses (*r += x and r.get_value()). */
#ifndef EG_SHIM_REDUCER_OPADD_H
#define EG_SHIM_REDUCER_OPADD_H
#include <atomic>
namespace cilk {
template <class T> class reducer_opadd {
    std::atomic<T> v_;
  public:
    struct view {
        std::atomic<T> *p;
        view &operator+=(T x) { p->fetch_add(x); return *this; }
    };
    explicit reducer_opadd(T init) : v_(init) {}
    view operator*() { return view{&v_}; }
    T get_value() const { return v_.load(); }
};
}  // namespace cilk
#endif
