/*
 * Kokkos_Core.hpp -- a minimal host-only stand-in for the parts of the
 * Kokkos API that the reference's damage kernel uses, so that its own
 * sources (src/kokkos_kernel.h, src/kokkos_host.cpp) compile unchanged
 * into oracle/_ref/ with a plain C++ compiler.
 *
 * TEST INFRASTRUCTURE ONLY: it serves the reference build that pins the
 * oracle's damage statement; nothing in the product includes it.
 *
 * What it provides, and with what meaning:
 *   - View<T*>: a reference-counted, zero-initialised 1-D array; operator()
 *     of a const view returns a mutable reference, as Kokkos views do;
 *     HostMirror is the same type; create_mirror_view allocates a view of
 *     the same length; deep_copy copies element by element.
 *   - TeamPolicy<> and its member_type: declared so the typedefs compile
 *     (the reference's parallel_for takes a plain count).
 *   - parallel_for(n, f): f(i) for i in [0, n), in contiguous chunks over
 *     shim_threads() host threads (1 by default, as the reference's
 *     kokkos_init_ asks for one thread).
 *   - initialize/finalize and InitArguments: no work.
 */
#ifndef XT_KOKKOS_SHIM_HPP
#define XT_KOKKOS_SHIM_HPP

#include <cstddef>
#include <memory>
#include <thread>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline

namespace Kokkos {

struct InitArguments {
    int num_threads = -1;
    int num_numa = -1;
    int device_id = -1;
};

inline int& shim_threads()
{
    static int n = 1;
    return n;
}

inline void initialize(const InitArguments&) {}
inline void finalize() {}

template <class DataType>
class View;

template <class T>
class View<T*> {
    std::shared_ptr<std::vector<T>> data_;

public:
    typedef View<T*> HostMirror;
    View() = default;
    View(const char*, std::size_t n) : data_(std::make_shared<std::vector<T>>(n, T())) {}
    T& operator()(std::size_t i) const { return (*data_)[i]; }
    std::size_t size() const { return data_ ? data_->size() : 0; }
};

template <class T>
View<T*> create_mirror_view(const View<T*>& v)
{
    return View<T*>("mirror", v.size());
}

template <class T>
void deep_copy(const View<T*>& dst, const View<T*>& src)
{
    for (std::size_t i = 0; i < src.size(); ++i) dst(i) = src(i);
}

template <class... P>
class TeamPolicy {
public:
    struct member_type {
        int league_rank() const { return 0; }
        int team_rank() const { return 0; }
        int team_size() const { return 1; }
    };
    TeamPolicy(int, int) {}
};

template <class F>
void parallel_for(int n, const F& f)
{
    const int nt = shim_threads() > 1 ? shim_threads() : 1;
    if (nt == 1 || n < 2 * nt) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> pool;
    const int chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) {
        const int b = t * chunk, e = (b + chunk < n) ? b + chunk : n;
        if (b >= e) break;
        pool.emplace_back([&f, b, e] {
            for (int i = b; i < e; ++i) f(i);
        });
    }
    for (auto& th : pool) th.join();
}

}  // namespace Kokkos

#endif
