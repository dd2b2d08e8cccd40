/*
 * TU/cu/Array++.h -- pitched 2D device arrays for the GB300 filter path.
 *
 * A minimal stand-in for the pitched device array the reference's filters
 * take (TU::cu::Array2 over TULibs' TU::array with cu::allocator,
 * TU/cu/Array++.h and TU/cu/allocator.h): rows aligned to 256 bytes, memory
 * zeroed at allocation, row iterators for the filters' convolve(ib, ie, out)
 * calls.  Owns its device memory (cudaMalloc / cudaFree); copying is explicit.
 */
#ifndef TUCU_CXX_ARRAY_H
#define TUCU_CXX_ARRAY_H

#include <cuda_runtime.h>

#include <cstddef>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace TU
{
namespace cu
{

/* An iterator over the rows of a pitched 2D image: what the filters read is
 * the row pointer, the pitch in bytes and the row length. */
template <class T>
class RowIterator
{
  public:
    using value_type = T;
    RowIterator() = default;
    RowIterator(T* row, size_t pitch, int cols) : row_(row), pitch_(pitch), cols_(cols) {}
    T* ptr() const { return row_; }
    size_t pitch() const { return pitch_; }
    int cols() const { return cols_; }
    RowIterator& operator++()
    {
        row_ = step(row_, (ptrdiff_t)pitch_);
        return *this;
    }
    RowIterator operator+(ptrdiff_t n) const { return RowIterator(step(row_, n * (ptrdiff_t)pitch_), pitch_, cols_); }
    ptrdiff_t operator-(const RowIterator& o) const
    {
        return (reinterpret_cast<const char*>(row_) - reinterpret_cast<const char*>(o.row_)) /
               (ptrdiff_t)pitch_;
    }
    bool operator==(const RowIterator& o) const { return row_ == o.row_; }
    bool operator!=(const RowIterator& o) const { return row_ != o.row_; }
    /* The const view of the same rows. */
    operator RowIterator<const T>() const { return RowIterator<const T>(row_, pitch_, cols_); }

  private:
    using Byte = typename std::conditional<std::is_const<T>::value, const char, char>::type;
    static T* step(T* p, ptrdiff_t bytes) { return reinterpret_cast<T*>(reinterpret_cast<Byte*>(p) + bytes); }

    T* row_ = nullptr;
    size_t pitch_ = 0;
    int cols_ = 0;
};

template <class T>
class Array2
{
  public:
    Array2() = default;
    Array2(int rows, int cols) { resize(rows, cols); }
    ~Array2() { release(); }
    Array2(const Array2&) = delete;
    Array2& operator=(const Array2&) = delete;
    Array2(Array2&& o) noexcept { swap(o); }
    Array2& operator=(Array2&& o) noexcept
    {
        swap(o);
        return *this;
    }

    /* Reallocates (contents zeroed); rows padded to a multiple of 256 bytes. */
    void resize(int rows, int cols)
    {
        if (rows < 0 || cols < 0)
            throw std::invalid_argument("Array2: negative size");
        release();
        rows_ = rows;
        cols_ = cols;
        pitch_ = ((size_t)cols * sizeof(T) + 255) / 256 * 256;
        if (rows && cols) {
            check(cudaMalloc(&data_, pitch_ * rows), "cudaMalloc");
            check(cudaMemset(data_, 0, pitch_ * rows), "cudaMemset");
        }
    }
    int nrow() const { return rows_; }
    int ncol() const { return cols_; }
    size_t pitch() const { return pitch_; }
    T* data() { return static_cast<T*>(data_); }
    const T* data() const { return static_cast<const T*>(data_); }

    RowIterator<T> begin() { return RowIterator<T>(data(), pitch_, cols_); }
    RowIterator<T> end() { return begin() + rows_; }
    RowIterator<const T> begin() const { return RowIterator<const T>(data(), pitch_, cols_); }
    RowIterator<const T> end() const { return begin() + rows_; }
    RowIterator<const T> cbegin() const { return begin(); }
    RowIterator<const T> cend() const { return end(); }

    /* Copies from / to a host image with `host_pitch` bytes per row. */
    void upload(const T* host, size_t host_pitch)
    {
        check(cudaMemcpy2D(data_, pitch_, host, host_pitch, (size_t)cols_ * sizeof(T), rows_,
                           cudaMemcpyHostToDevice),
              "cudaMemcpy2D");
    }
    void download(T* host, size_t host_pitch) const
    {
        check(cudaMemcpy2D(host, host_pitch, data_, pitch_, (size_t)cols_ * sizeof(T), rows_,
                           cudaMemcpyDeviceToHost),
              "cudaMemcpy2D");
    }

  private:
    static void check(cudaError_t e, const char* what)
    {
        if (e != cudaSuccess)
            throw std::runtime_error(std::string("Array2: ") + what + ": " + cudaGetErrorString(e));
    }
    void release()
    {
        if (data_)
            cudaFree(data_);
        data_ = nullptr;
        rows_ = cols_ = 0;
        pitch_ = 0;
    }
    void swap(Array2& o)
    {
        std::swap(data_, o.data_);
        std::swap(rows_, o.rows_);
        std::swap(cols_, o.cols_);
        std::swap(pitch_, o.pitch_);
    }

    void* data_ = nullptr;
    int rows_ = 0, cols_ = 0;
    size_t pitch_ = 0;
};

/* An iterator over the slices of a pitched 3D array (slices of rows x cols):
 * the first slice's row pointer, the row pitch and the slice pitch in bytes. */
template <class T>
class SliceIterator
{
  public:
    SliceIterator(T* p, size_t pitch, size_t slice_pitch, int rows, int cols)
        : p_(p), pitch_(pitch), slice_pitch_(slice_pitch), rows_(rows), cols_(cols)
    {
    }
    T* ptr() const { return p_; }
    size_t pitch() const { return pitch_; }
    size_t slice_pitch() const { return slice_pitch_; }
    int rows() const { return rows_; }
    int cols() const { return cols_; }

  private:
    T* p_;
    size_t pitch_, slice_pitch_;
    int rows_, cols_;
};

/* A pitched 3D device array of `slices` images of rows x cols (the
 * reference's cu::Array3 in the layout its stereo code uses with
 * DISPARITY_MAJOR): rows aligned to 256 bytes, memory zeroed at allocation. */
template <class T>
class Array3
{
  public:
    Array3(int slices, int rows, int cols) : slices_(slices)
    {
        if (slices < 0)
            throw std::invalid_argument("Array3: negative size");
        planes_.resize(slices > 0 ? 1 : 0);
        if (slices > 0) {
            // one allocation: slices stacked as rows of one tall Array2
            planes_[0].resize(slices * rows, cols);
        }
        rows_ = rows;
        cols_ = cols;
    }
    int size() const { return slices_; }
    int nrow() const { return rows_; }
    int ncol() const { return cols_; }
    size_t pitch() const { return slices_ ? planes_[0].pitch() : 0; }
    size_t slice_pitch() const { return pitch() * rows_; }
    SliceIterator<T> begin()
    {
        return SliceIterator<T>(slices_ ? planes_[0].data() : nullptr, pitch(), slice_pitch(), rows_, cols_);
    }
    SliceIterator<const T> cbegin() const
    {
        return SliceIterator<const T>(slices_ ? planes_[0].data() : nullptr, pitch(), slice_pitch(), rows_, cols_);
    }
    /* Slice d as rows of a 2D image. */
    RowIterator<T> slice(int d)
    {
        return RowIterator<T>(planes_[0].data(), pitch(), cols_) + (ptrdiff_t)d * rows_;
    }
    /* Copies every slice to a host buffer of slices x rows x cols. */
    void download(T* host) const
    {
        if (slices_)
            planes_[0].download(host, (size_t)cols_ * sizeof(T));
    }

  private:
    int slices_ = 0, rows_ = 0, cols_ = 0;
    std::vector<Array2<T>> planes_;
};

}  // namespace cu
}  // namespace TU

#endif
