// Minimal host containers standing in for TULibs' TU::Array / TU::Array2
// (only what the reference code compiled by oracle/Makefile touches).
#pragma once
#include <cstddef>
#include <vector>

namespace TU
{
template <class T, size_t N = 0>
class Array
{
  public:
    Array() = default;
    explicit Array(size_t n) : _v(n) {}
    void resize(size_t n) { _v.resize(n); }
    size_t size() const { return _v.size(); }
    T& operator[](size_t i) { return _v[i]; }
    const T& operator[](size_t i) const { return _v[i]; }
    T* data() { return _v.data(); }
    const T* data() const { return _v.data(); }
    Array& operator=(const T& c)
    {
        for (auto& x : _v) x = c;
        return *this;
    }

  private:
    std::vector<T> _v;
};

// ROW is the row type (e.g. Array<float>), as in TULibs.
template <class ROW, size_t R = 0, size_t C = 0>
class Array2
{
  public:
    Array2() = default;
    Array2(size_t r, size_t c) { resize(r, c); }
    void resize(size_t r, size_t c)
    {
        _rows.assign(r, ROW());
        for (auto& row : _rows) row.resize(c);
        _ncol = c;
    }
    size_t nrow() const { return _rows.size(); }
    size_t ncol() const { return _ncol; }
    ROW& operator[](size_t i) { return _rows[i]; }
    const ROW& operator[](size_t i) const { return _rows[i]; }
    Array2& operator=(int c)
    {
        for (auto& row : _rows) row = c;
        return *this;
    }

  private:
    std::vector<ROW> _rows;
    size_t _ncol = 0;
};
}  // namespace TU
