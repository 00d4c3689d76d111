// cereal/access.hpp - stand-in for the part of cereal 1.3 that the
// reference's Graph::save / Graph::load (include/spoa/graph.hpp:187-276)
// use, and two in-memory binary archives to drive them.
//
// TEST INFRASTRUCTURE ONLY: lets oracle/Makefile compile the reference's
// own serialisation code into oracle/_ref/spoa_ref_driver_cereal (cereal
// is fetched by the reference's CMake build and is not part of its tree).
// Restated from cereal's published interface: access::construct / member
// serialize through `friend cereal::access`, archive(...) over values,
// std::vector, std::pair and std::unique_ptr, classes with a serialize
// member or save/load members, CEREAL_NVP as a plain value.
#ifndef ORACLE_SHIM_CEREAL_ACCESS_HPP_
#define ORACLE_SHIM_CEREAL_ACCESS_HPP_

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define CEREAL_NVP(x) x

namespace cereal {

class access {
 public:
  template <class T>
  static T* construct() { return new T(); }
  template <class A, class T>
  static auto serialize(A& a, T& t) -> decltype(t.serialize(a), void()) { t.serialize(a); }
  template <class A, class T>
  static auto save(A& a, const T& t) -> decltype(t.save(a), void()) { t.save(a); }
  template <class A, class T>
  static auto load(A& a, T& t) -> decltype(t.load(a), void()) { t.load(a); }
};

class BinaryOutputArchive {
 public:
  explicit BinaryOutputArchive(std::string* out) : out_(out) {}
  template <class... T>
  void operator()(T&&... v) {
    int unused[] = {0, (Put(v), 0)...};
    (void)unused;
  }

 private:
  template <class T>
  typename std::enable_if<std::is_arithmetic<T>::value>::type Put(const T& v) {
    out_->append(reinterpret_cast<const char*>(&v), sizeof(v));
  }
  template <class T>
  void Put(const std::vector<T>& v) {
    Put(static_cast<std::uint64_t>(v.size()));
    for (const auto& x : v) Put(x);
  }
  template <class A, class B>
  void Put(const std::pair<A, B>& v) {
    Put(v.first);
    Put(v.second);
  }
  template <class T>
  void Put(const std::unique_ptr<T>& v) {
    Put(static_cast<std::uint8_t>(v ? 1 : 0));
    if (v) Put(*v);
  }
  template <class T>
  auto Put(const T& v) -> decltype(access::save(*this, v), void()) {
    access::save(*this, v);
  }
  template <class T>
  auto Put(const T& v) -> decltype(access::serialize(*this, const_cast<T&>(v)), void()) {
    access::serialize(*this, const_cast<T&>(v));
  }

  std::string* out_;
};

class BinaryInputArchive {
 public:
  explicit BinaryInputArchive(const std::string& in) : in_(in) {}
  template <class... T>
  void operator()(T&&... v) {
    int unused[] = {0, (Get(v), 0)...};
    (void)unused;
  }

 private:
  template <class T>
  typename std::enable_if<std::is_arithmetic<T>::value>::type Get(T& v) {
    if (pos_ + sizeof(v) > in_.size()) throw std::runtime_error("archive: out of data");
    std::memcpy(&v, in_.data() + pos_, sizeof(v));
    pos_ += sizeof(v);
  }
  template <class T>
  void Get(std::vector<T>& v) {
    std::uint64_t n = 0;
    Get(n);
    v.clear();
    v.resize(n);
    for (auto& x : v) Get(x);
  }
  template <class A, class B>
  void Get(std::pair<A, B>& v) {
    Get(v.first);
    Get(v.second);
  }
  template <class T>
  void Get(std::unique_ptr<T>& v) {
    std::uint8_t has = 0;
    Get(has);
    v.reset();
    if (has) {
      v.reset(access::construct<T>());
      Get(*v);
    }
  }
  template <class T>
  auto Get(T& v) -> decltype(access::load(*this, v), void()) {
    access::load(*this, v);
  }
  template <class T>
  auto Get(T& v) -> decltype(access::serialize(*this, v), void()) {
    access::serialize(*this, v);
  }

  const std::string& in_;
  std::size_t pos_ = 0;
};

}  // namespace cereal

#endif  // ORACLE_SHIM_CEREAL_ACCESS_HPP_
