// intp::Mesh / intp::MeshDimension for the GB300 library's C++ drop-in.
//
// Same interface as the reference's src/include/Mesh.hpp (MeshDimension
// :11-116, Mesh :125-383): an N-d row-major array (last index fastest) with
// per-axis strided iterators. Values live in host memory; the interpolation
// functions upload them to the GPU.
#ifndef INTP_GPU_MESH_HPP
#define INTP_GPU_MESH_HPP

#include <algorithm>
#include <array>
#include <cstddef>
#include <iterator>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace intp {

template <std::size_t D>
class MeshDimension {
   public:
    using size_type = std::size_t;
    static constexpr size_type dim = D;
    using index_type = std::array<size_type, D>;

    MeshDimension() = default;
    MeshDimension(index_type sizes) : sizes_(sizes) {}
    template <typename... Args, typename = typename std::enable_if<sizeof...(Args) == D>::type>
    MeshDimension(Args... args) : sizes_{static_cast<size_type>(args)...} {}
    MeshDimension(size_type n) { sizes_.fill(n); }

    size_type size() const {
        size_type s = 1;
        for (auto v : sizes_) s *= v;
        return s;
    }
    size_type dim_size(size_type d) const { return sizes_[d]; }
    size_type& dim_size(size_type d) { return sizes_[d]; }
    // product of the last `d` axis sizes (stride of axis D-1-d)
    size_type dim_acc_size(size_type d) const {
        size_type s = 1;
        for (size_type k = 0; k < d; ++k) s *= sizes_[D - 1 - k];
        return s;
    }
    operator index_type() const { return sizes_; }

    size_type indexing(const index_type& idx) const {
        size_type lin = 0;
        for (size_type d = 0; d < D; ++d) lin = lin * sizes_[d] + idx[d];
        return lin;
    }
    template <typename... Indices>
    size_type indexing_safe(Indices... indices) const {
        return indexing_safe(index_type{static_cast<size_type>(indices)...});
    }
    size_type indexing_safe(const index_type& idx) const {
#if defined(INTP_ENABLE_ASSERTION) || defined(INTP_DEBUG)
        for (size_type d = 0; d < D; ++d)
            if (idx[d] >= sizes_[d])
                throw std::runtime_error("Mesh access out of range at dim " + std::to_string(d));
#endif
        return indexing(idx);
    }
    index_type dimwise_indices(size_type lin) const {
        index_type idx{};
        for (size_type k = 0; k < D; ++k) {
            const size_type d = D - 1 - k;
            idx[d] = lin % sizes_[d];
            lin /= sizes_[d];
        }
        return idx;
    }
    void resize(index_type sizes) { sizes_ = sizes; }

   private:
    index_type sizes_{};
};

template <typename T, std::size_t D, typename Alloc = std::allocator<T>>
class Mesh {
   public:
    using size_type = std::size_t;
    using val_type = T;
    static const size_type dim = D;
    using index_type = typename MeshDimension<D>::index_type;
    using allocator_type = Alloc;

   private:
    using container_type = std::vector<T, Alloc>;

    // random-access iterator stepping by a fixed stride
    template <typename U>
    class skip_iterator {
       public:
        using value_type = typename std::remove_const<U>::type;
        using difference_type = std::ptrdiff_t;
        using pointer = U*;
        using reference = U&;
        using iterator_category = std::random_access_iterator_tag;

        skip_iterator(U* p, difference_type step) : p_(p), step_(step) {}
        operator skip_iterator<const U>() const { return {p_, step_}; }
        explicit operator const U*() const { return p_; }
        reference operator*() const { return *p_; }
        pointer operator->() const { return p_; }
        reference operator[](difference_type n) const { return p_[n * step_]; }
        skip_iterator& operator++() { p_ += step_; return *this; }
        skip_iterator operator++(int) { auto t = *this; p_ += step_; return t; }
        skip_iterator& operator--() { p_ -= step_; return *this; }
        skip_iterator operator--(int) { auto t = *this; p_ -= step_; return t; }
        skip_iterator& operator+=(difference_type n) { p_ += n * step_; return *this; }
        skip_iterator& operator-=(difference_type n) { p_ -= n * step_; return *this; }
        skip_iterator operator+(difference_type n) const { auto t = *this; return t += n; }
        skip_iterator operator-(difference_type n) const { auto t = *this; return t -= n; }
        friend skip_iterator operator+(difference_type n, skip_iterator it) { return it += n; }
        difference_type operator-(const skip_iterator& o) const { return (p_ - o.p_) / step_; }
        bool operator==(const skip_iterator& o) const { return p_ == o.p_ && step_ == o.step_; }
        bool operator!=(const skip_iterator& o) const { return !(*this == o); }
        bool operator<(const skip_iterator& o) const { return o - *this > 0; }
        bool operator>(const skip_iterator& o) const { return o < *this; }
        bool operator<=(const skip_iterator& o) const { return !(*this > o); }
        bool operator>=(const skip_iterator& o) const { return !(*this < o); }

       private:
        U* p_;
        difference_type step_;
    };

   public:
    explicit Mesh(const MeshDimension<D>& dims, const Alloc& alloc = Alloc())
        : storage_(alloc), dims_(dims) {
        storage_.resize(dims_.size(), T{});
    }
    explicit Mesh(size_type n, const Alloc& alloc = Alloc()) : Mesh(MeshDimension<D>(n), alloc) {}
    template <typename... Args, typename = typename std::enable_if<sizeof...(Args) == D>::type,
              typename = typename std::enable_if<
                  std::is_integral<typename std::common_type<Args...>::type>::value>::type>
    explicit Mesh(Args... args) : Mesh(MeshDimension<D>(static_cast<size_type>(args)...)) {}
    template <typename InputIter,
              typename = typename std::enable_if<
                  D == 1u && std::is_convertible<typename std::iterator_traits<InputIter>::iterator_category,
                                                 std::input_iterator_tag>::value>::type>
    explicit Mesh(std::pair<InputIter, InputIter> range, const Alloc& alloc = Alloc())
        : storage_(range.first, range.second, alloc), dims_{static_cast<size_type>(storage_.size())} {}
    template <typename A2>
    Mesh(const Mesh<T, D, A2>& other, const Alloc& alloc = Alloc()) : Mesh(other.dimension(), alloc) {
        std::copy(other.begin(), other.end(), storage_.begin());
    }

    size_type size() const { return storage_.size(); }
    size_type dim_size(size_type d) const { return dims_.dim_size(d); }
    const MeshDimension<D>& dimension() const { return dims_; }
    void resize(index_type sizes) {
        dims_.resize(sizes);
        storage_.resize(dims_.size());
    }

    template <typename... Indices>
    T& operator()(Indices... idx) {
        return storage_[dims_.indexing_safe(idx...)];
    }
    template <typename... Indices>
    const T& operator()(Indices... idx) const {
        return storage_[dims_.indexing_safe(idx...)];
    }
    T& operator()(index_type idx) { return storage_[dims_.indexing(idx)]; }
    const T& operator()(index_type idx) const { return storage_[dims_.indexing(idx)]; }
    const T* data() const { return storage_.data(); }
    T* data() { return storage_.data(); }

    typename container_type::const_iterator begin() const { return storage_.cbegin(); }
    typename container_type::const_iterator end() const { return storage_.cend(); }

    skip_iterator<T> begin(size_type d, index_type idx) {
        idx[d] = 0;
        return {storage_.data() + dims_.indexing_safe(idx), stride(d)};
    }
    skip_iterator<T> end(size_type d, index_type idx) {
        idx[d] = dims_.dim_size(d);
        return {storage_.data() + dims_.indexing(idx), stride(d)};
    }
    skip_iterator<const T> begin(size_type d, index_type idx) const {
        idx[d] = 0;
        return {storage_.data() + dims_.indexing_safe(idx), stride(d)};
    }
    skip_iterator<const T> end(size_type d, index_type idx) const {
        idx[d] = dims_.dim_size(d);
        return {storage_.data() + dims_.indexing(idx), stride(d)};
    }
    index_type iter_indices(typename container_type::const_iterator it) const {
        return dims_.dimwise_indices(static_cast<size_type>(std::distance(begin(), it)));
    }
    index_type iter_indices(skip_iterator<const T> it) const {
        return dims_.dimwise_indices(
            static_cast<size_type>(static_cast<const T*>(it) - storage_.data()));
    }

   private:
    std::ptrdiff_t stride(size_type d) const {
        return static_cast<std::ptrdiff_t>(dims_.dim_acc_size(D - d - 1));
    }
    container_type storage_;
    MeshDimension<D> dims_;
};

}  // namespace intp

#endif
