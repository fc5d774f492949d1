// intp::InterpolationFunction and friends: header-only C++ drop-in for the
// reference library's interface (src/include/Interpolation.hpp,
// InterpolationTemplate.hpp), backed by the GB300 CUDA library through its
// C-ABI (include/intp_gpu.h). Link with libintp_gb300.so.
//
// Same class templates, constructors, methods and exceptions as the
// reference; semantics are those of the reference built with
// INTP_PERIODIC_NO_DUMMY_POINT. Per-point calls are correct but each is a
// device round trip; the batch methods (evaluate / evaluate_device) are the
// fast path. The compute precision defaults to FP64 (parity with the
// reference); intp::gpu::set_default_precision(intp::gpu::Precision::mixed)
// or -DINTP_GPU_DEFAULT_MIXED selects the FP32 mixed form for tables built
// afterwards.
#ifndef INTP_GPU_INTERPOLATION_HPP
#define INTP_GPU_INTERPOLATION_HPP

#include <array>
#include <cmath>
#include <cstdint>
#include <iterator>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "../intp_gpu.h"
#include "Mesh.hpp"

namespace intp {

namespace gpu {

enum class Precision { fp64 = INTP_PRECISION_FP64, mixed = INTP_PRECISION_MIXED };

inline Precision& default_precision_ref() {
#ifdef INTP_GPU_DEFAULT_MIXED
    static thread_local Precision p = Precision::mixed;
#else
    static thread_local Precision p = Precision::fp64;
#endif
    return p;
}
inline void set_default_precision(Precision p) { default_precision_ref() = p; }
inline Precision default_precision() { return default_precision_ref(); }

// Maps a C-ABI status onto the reference's exception types.
inline void check(intp_status s) {
    if (s == INTP_OK) return;
    const std::string msg = intp_last_error();
    switch (s) {
        case INTP_ERR_DOMAIN: throw std::domain_error(msg);
        case INTP_ERR_OUT_OF_MEMORY: throw std::bad_alloc();
        default: throw std::runtime_error(msg);
    }
}

struct TableDeleter {
    void operator()(intp_table* t) const { intp_table_destroy(t); }
};
using TablePtr = std::shared_ptr<intp_table>;

}  // namespace gpu

// How a value type T crosses the C-ABI: `channels` doubles per value, channel
// fastest. Arithmetic types are one channel and std::array<V, N> is N (a
// vector-valued function, as the reference interpolates Vec<N, T> values,
// test/src/interpolation-test.cpp "interpolation on vector"). Specialise it
// for other vector types.
template <typename T, typename = void>
struct value_traits {
    static constexpr std::size_t channels = 1;
    static double get(const T& v, std::size_t) { return static_cast<double>(v); }
    static void set(T& v, std::size_t, double x) { v = static_cast<T>(x); }
};

template <typename V, std::size_t N>
struct value_traits<std::array<V, N>> {
    static constexpr std::size_t channels = N;
    static double get(const std::array<V, N>& v, std::size_t c) { return static_cast<double>(v[c]); }
    static void set(std::array<V, N>& v, std::size_t c, double x) { v[c] = static_cast<V>(x); }
};

namespace detail {

template <typename T>
struct is_iter_pair_arg {
    template <typename U>
    static auto test(int) -> decltype(typename std::iterator_traits<U>::iterator_category{}, std::true_type{});
    template <typename>
    static std::false_type test(...);
    static constexpr bool value = decltype(test<T>(0))::value && !std::is_arithmetic<T>::value;
};

// fills one axis of the table description from a range argument
template <typename T_>
typename std::enable_if<std::is_arithmetic<T_>::value>::type axis_arg(
    intp_table_desc& d, std::vector<std::vector<double>>&, std::size_t axis, std::pair<T_, T_> r) {
    d.range_lo[axis] = static_cast<double>(r.first);
    d.range_hi[axis] = static_cast<double>(r.second);
    d.coords[axis] = nullptr;
}

template <typename T_>
typename std::enable_if<is_iter_pair_arg<T_>::value>::type axis_arg(
    intp_table_desc& d, std::vector<std::vector<double>>& keep, std::size_t axis, std::pair<T_, T_> r) {
    keep[axis].clear();
    for (auto it = r.first; it != r.second; ++it) keep[axis].push_back(static_cast<double>(*it));
    d.coords[axis] = keep[axis].data();
}

}  // namespace detail

template <typename T, std::size_t D, std::size_t O, typename U = double>
class InterpolationFunctionTemplate;

// Read-only view of the spline behind an interpolation function
// (the subset of BSpline, src/include/BSpline.hpp:32-760, callers inspect).
template <typename T, std::size_t D, std::size_t O, typename U>
class SplineView {
   public:
    using size_type = std::size_t;
    using knot_type = U;
    using KnotContainer = std::vector<U>;
    static constexpr size_type dim = D;
    static constexpr size_type order = O;

    explicit SplineView(gpu::TablePtr t = nullptr) : table_(std::move(t)) { load(); }

    size_type knots_num(size_type d) const { return knots_[d].size(); }
    typename KnotContainer::const_iterator knots_begin(size_type d) const { return knots_[d].cbegin(); }
    typename KnotContainer::const_iterator knots_end(size_type d) const { return knots_[d].cend(); }
    const std::pair<U, U>& range(size_type d) const { return range_[d]; }
    bool periodicity(size_type d) const { return periodic_[d]; }
    static constexpr size_type get_order() { return O; }
    // control points, row-major, copied from the device
    Mesh<T, D> control_points() const {
        using VT = value_traits<T>;
        std::array<std::size_t, D> dims{};
        for (size_type d = 0; d < D; ++d) dims[d] = ncp_[d];
        Mesh<T, D> m{MeshDimension<D>(dims)};
        std::vector<double> buf(m.size() * VT::channels);
        gpu::check(intp_table_get_control_points(table_.get(), buf.data()));
        for (std::size_t i = 0; i < m.size(); ++i) {
            T& v = m(m.dimension().dimwise_indices(i));
            for (std::size_t c = 0; c < VT::channels; ++c) VT::set(v, c, buf[i * VT::channels + c]);
        }
        return m;
    }

   private:
    friend class InterpolationFunctionTemplate<T, D, O, U>;
    template <typename, std::size_t, std::size_t, typename>
    friend class InterpolationFunction;
    void load() {
        if (!table_) return;
        for (size_type d = 0; d < D; ++d) {
            int64_t nk = 0;
            double lo = 0, hi = 0;
            int32_t per = 0, uni = 0;
            gpu::check(intp_table_axis_info(table_.get(), static_cast<int32_t>(d), &nk, &lo, &hi, &per, &uni));
            std::vector<double> k(static_cast<std::size_t>(nk));
            gpu::check(intp_table_knots(table_.get(), static_cast<int32_t>(d), k.data()));
            knots_[d].assign(k.begin(), k.end());
            range_[d] = {static_cast<U>(lo), static_cast<U>(hi)};
            periodic_[d] = per != 0;
            uniform_[d] = uni != 0;
        }
    }
    gpu::TablePtr table_;
    std::array<KnotContainer, D> knots_{};
    std::array<std::pair<U, U>, D> range_{};
    std::array<bool, D> periodic_{};
    std::array<bool, D> uniform_{};
    std::array<std::size_t, D> ncp_{};
};

template <typename T, std::size_t D, std::size_t O, typename U = double>
class InterpolationFunction {
   public:
    using spline_type = SplineView<T, D, O, U>;
    using val_type = T;
    using size_type = std::size_t;
    using coord_type = U;
    using diff_type = std::ptrdiff_t;
    static constexpr size_type dim = D;
    static constexpr size_type order = O;
    template <typename T_>
    using DimArray = std::array<T_, D>;

    friend class InterpolationFunctionTemplate<T, D, O, U>;

    // 1D: (periodic, f_range, x_range) and (f_range, x_range),
    // Interpolation.hpp:49-79
    template <typename InputIter, typename C1, typename C2,
              typename std::enable_if<D == 1u && std::is_convertible<
                                                     typename std::iterator_traits<InputIter>::iterator_category,
                                                     std::input_iterator_tag>::value>::type* = nullptr>
    InterpolationFunction(bool periodic, std::pair<InputIter, InputIter> f_range, std::pair<C1, C2> x_range)
        : InterpolationFunction(DimArray<bool>{{periodic}}, Mesh<val_type, 1u>{std::make_pair(f_range.first, f_range.second)},
                                static_cast<std::pair<typename std::common_type<C1, C2>::type,
                                                      typename std::common_type<C1, C2>::type>>(x_range)) {}

    template <typename InputIter, typename C1, typename C2,
              typename std::enable_if<D == 1u && std::is_convertible<
                                                     typename std::iterator_traits<InputIter>::iterator_category,
                                                     std::input_iterator_tag>::value>::type* = nullptr>
    InterpolationFunction(std::pair<InputIter, InputIter> f_range, std::pair<C1, C2> x_range)
        : InterpolationFunction(false, f_range, x_range) {}

    // nD: (periodicity, mesh, x_ranges...), Interpolation.hpp:92-107
    template <typename... Ts>
    InterpolationFunction(DimArray<bool> periodicity, const Mesh<val_type, D>& f_mesh, std::pair<Ts, Ts>... x_ranges)
        : InterpolationFunction(InterpolationFunctionTemplate<T, D, O, U>(periodicity, f_mesh.dimension(), x_ranges...)
                                    .interpolate(f_mesh)) {}

    template <typename... Ts>
    InterpolationFunction(const Mesh<val_type, D>& f_mesh, std::pair<Ts, Ts>... x_ranges)
        : InterpolationFunction(DimArray<bool>{}, f_mesh, x_ranges...) {}

    InterpolationFunction() = default;

    // -- evaluation, Interpolation.hpp:132-244 --
    template <typename... Coords, typename = typename std::enable_if<std::is_arithmetic<
                                      typename std::common_type<Coords...>::type>::value>::type>
    val_type operator()(Coords... x) const {
        return eval_one(DimArray<coord_type>{static_cast<coord_type>(x)...}, nullptr);
    }
    val_type operator()(DimArray<coord_type> c) const { return eval_one(c, nullptr); }

    val_type at(DimArray<coord_type> c) const {
        boundary_check_(c);
        return eval_one(c, nullptr);
    }
    template <typename... Coords, typename = typename std::enable_if<std::is_arithmetic<
                                      typename std::common_type<Coords...>::type>::value>::type>
    val_type at(Coords... x) const {
        return at(DimArray<coord_type>{static_cast<coord_type>(x)...});
    }

    val_type derivative(DimArray<coord_type> c, DimArray<size_type> k) const {
        int32_t kk[D];
        for (size_type d = 0; d < D; ++d) kk[d] = static_cast<int32_t>(k[d]);
        return eval_one(c, kk);
    }
    template <typename... Args>
    val_type derivative(DimArray<coord_type> c, Args... k) const {
        return derivative(c, DimArray<size_type>{static_cast<size_type>(k)...});
    }
    template <typename... Pairs>
    val_type derivative(Pairs... p) const {
        return derivative(DimArray<coord_type>{static_cast<coord_type>(p.first)...},
                          DimArray<size_type>{static_cast<size_type>(p.second)...});
    }
    val_type derivative_at(DimArray<coord_type> c, DimArray<size_type> k) const {
        boundary_check_(c);
        return derivative(c, k);
    }
    template <typename... Args>
    val_type derivative_at(DimArray<coord_type> c, Args... k) const {
        return derivative_at(c, DimArray<size_type>{static_cast<size_type>(k)...});
    }
    template <typename... Pairs>
    val_type derivative_at(Pairs... p) const {
        return derivative_at(DimArray<coord_type>{static_cast<coord_type>(p.first)...},
                             DimArray<size_type>{static_cast<size_type>(p.second)...});
    }

    // -- batch evaluation (the fast path) --
    // Host buffers: coords n x D, out n x nderiv x C with C =
    // value_traits<T>::channels (derivs nderiv x D, or nullptr for values).
    void evaluate(const double* coords, std::size_t n, double* out, const int32_t* derivs = nullptr,
                  int32_t nderiv = 1) const {
        gpu::check(intp_eval_host(table_.get(), coords, static_cast<int64_t>(n), derivs, nderiv, out, INTP_F64, nullptr));
    }
    // Device buffers on `stream` (out_dtype INTP_F64 or INTP_F32).
    void evaluate_device(const double* coords, std::size_t n, void* out, int32_t out_dtype,
                         const int32_t* derivs = nullptr, int32_t nderiv = 1, void* stream = nullptr) const {
        gpu::check(intp_eval(table_.get(), coords, static_cast<int64_t>(n), derivs, nderiv, out, out_dtype, stream));
    }

    // -- properties, Interpolation.hpp:248-267 --
    bool periodicity(size_type d) const { return spline_.periodicity(d); }
    bool uniform(size_type d) const { return spline_.uniform_[d]; }
    const std::pair<coord_type, coord_type>& range(size_type d) const { return spline_.range(d); }
    const spline_type& spline() const { return spline_; }
    static constexpr size_type get_order() { return O; }
    intp_table* handle() const { return table_.get(); }

   private:
    gpu::TablePtr table_;
    spline_type spline_;

    void attach(gpu::TablePtr t, const std::array<std::size_t, D>& ncp) {
        table_ = std::move(t);
        spline_ = spline_type(table_);
        spline_.ncp_ = ncp;
    }

    val_type eval_one(const DimArray<coord_type>& c, const int32_t* k) const {
        using VT = value_traits<T>;
        double x[D];
        for (size_type d = 0; d < D; ++d) x[d] = static_cast<double>(c[d]);
        double r[VT::channels] = {};
        gpu::check(intp_eval_host(table_.get(), x, 1, k, 1, r, INTP_F64, nullptr));
        val_type v{};
        for (std::size_t ch = 0; ch < VT::channels; ++ch) VT::set(v, ch, r[ch]);
        return v;
    }

    // Interpolation.hpp:482-491
    void boundary_check_(const DimArray<coord_type>& c) const {
        for (size_type d = 0; d < D; ++d)
            if (!periodicity(d) && (c[d] < range(d).first || c[d] > range(d).second))
                throw std::domain_error("Given coordinate out of interpolation function range!");
    }
};

// Knots and factors for a mesh shape; interpolate() solves control points
// for any value mesh of that shape (InterpolationTemplate.hpp:32-581).
template <typename T, std::size_t D, std::size_t O, typename U>
class InterpolationFunctionTemplate {
   public:
    using function_type = InterpolationFunction<T, D, O, U>;
    using size_type = std::size_t;
    using coord_type = U;
    using val_type = T;
    static constexpr size_type dim = D;
    static constexpr size_type order = O;
    template <typename V>
    using DimArray = std::array<V, D>;
    using MeshDim = MeshDimension<D>;

    template <typename... Ts>
    InterpolationFunctionTemplate(DimArray<bool> periodicity, MeshDim dims, std::pair<Ts, Ts>... x_ranges)
        : desc_{}, keep_(D) {
        static_assert(sizeof...(Ts) == D, "one x range per dimension");
        desc_.dim = static_cast<int32_t>(D);
        desc_.order = static_cast<int32_t>(O);
        desc_.precision = static_cast<int32_t>(gpu::default_precision());
        desc_.refine_steps = -1;
        desc_.channels = static_cast<int32_t>(value_traits<T>::channels);
        for (size_type d = 0; d < D; ++d) {
            desc_.periodic[d] = periodicity[d] ? 1 : 0;
            desc_.size[d] = static_cast<int64_t>(dims.dim_size(d));
            ncp_[d] = dims.dim_size(d);
        }
        size_type axis = 0;
        (void)std::initializer_list<int>{(detail::axis_arg(desc_, keep_, axis++, x_ranges), 0)...};
        // validate once (throws the reference's exception types)
        intp_table* t = nullptr;
        gpu::check(intp_table_create(&desc_, &t));
        proto_ = gpu::TablePtr(t, gpu::TableDeleter{});
    }
    template <typename C1, typename C2>
    InterpolationFunctionTemplate(bool periodicity, size_type f_length, std::pair<C1, C2> x_range)
        : InterpolationFunctionTemplate(DimArray<bool>{{periodicity}}, MeshDim{f_length}, x_range) {}
    template <typename C1, typename C2>
    InterpolationFunctionTemplate(size_type f_length, std::pair<C1, C2> x_range)
        : InterpolationFunctionTemplate(false, f_length, x_range) {}
    template <typename... Ts>
    InterpolationFunctionTemplate(MeshDim dims, std::pair<Ts, Ts>... x_ranges)
        : InterpolationFunctionTemplate(DimArray<bool>{}, dims, x_ranges...) {}

    // InterpolationTemplate.hpp:118-143
    function_type interpolate(const Mesh<val_type, D>& mesh) const {
        function_type f;
        interpolate(f, mesh);
        return f;
    }
    template <typename InputIter>
    function_type interpolate(std::pair<InputIter, InputIter> range) const {
        return interpolate(Mesh<val_type, D>{range});
    }
    void interpolate(function_type& f, const Mesh<val_type, D>& mesh) const {
        for (size_type d = 0; d < D; ++d)
            if (mesh.dim_size(d) != ncp_[d]) throw std::runtime_error("mesh shape does not match the template");
        intp_table* t = nullptr;
        gpu::check(intp_table_create(&desc_, &t));
        gpu::TablePtr tp(t, gpu::TableDeleter{});
        using VT = value_traits<T>;
        std::vector<double> v(mesh.size() * VT::channels);
        for (size_type i = 0; i < mesh.size(); ++i) {
            const T& x = mesh(mesh.dimension().dimwise_indices(i));
            for (std::size_t c = 0; c < VT::channels; ++c) v[i * VT::channels + c] = VT::get(x, c);
        }
        gpu::check(intp_table_interpolate(tp.get(), v.data(), 0, nullptr));
        gpu::check(intp_stream_synchronize(nullptr));
        f.attach(std::move(tp), ncp_);
    }

   private:
    intp_table_desc desc_;
    std::vector<std::vector<double>> keep_;
    std::array<std::size_t, D> ncp_{};
    gpu::TablePtr proto_;
};

// Interpolation.hpp:509-540
template <std::size_t O = std::size_t{3}, typename T = double, typename U = double>
class InterpolationFunction1D : public InterpolationFunction<T, std::size_t{1}, O, U> {
    using base = InterpolationFunction<T, std::size_t{1}, O, U>;

   public:
    template <typename InputIter>
    InterpolationFunction1D(std::pair<InputIter, InputIter> f_range, bool periodicity = false)
        : InterpolationFunction1D(
              std::make_pair(typename base::coord_type{},
                             static_cast<typename base::coord_type>(
                                 std::distance(f_range.first, f_range.second) - (periodicity ? 0 : 1))),
              f_range, periodicity) {}
    template <typename C1, typename C2, typename InputIter>
    InterpolationFunction1D(std::pair<C1, C2> x_range, std::pair<InputIter, InputIter> f_range,
                            bool periodicity = false)
        : base(periodicity, f_range, x_range) {}
};

// InterpolationTemplate.hpp:583-604
template <std::size_t O, typename T = double, typename U = double>
class InterpolationFunctionTemplate1D : public InterpolationFunctionTemplate<T, std::size_t{1}, O, U> {
    using base = InterpolationFunctionTemplate<T, std::size_t{1}, O, U>;

   public:
    InterpolationFunctionTemplate1D(typename base::size_type f_length, bool periodicity = false)
        : InterpolationFunctionTemplate1D(
              std::make_pair(typename base::coord_type{}, static_cast<typename base::coord_type>(f_length - 1)),
              f_length, periodicity) {}
    template <typename C1, typename C2>
    InterpolationFunctionTemplate1D(std::pair<C1, C2> x_range, typename base::size_type f_length,
                                    bool periodicity = false)
        : base(periodicity, f_length, x_range) {}
};

}  // namespace intp

#endif
