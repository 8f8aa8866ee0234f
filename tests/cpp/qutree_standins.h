// qutree_standins.h -- the few QuTree types the GpuSweep shim touches, cut
// down to the members it calls, so that the shim compiles and runs outside
// QuTree exactly as written for it.  Names and semantics follow the
// reference:
//   TensorShape   include/Core/TensorShape.h:44-61 (order, operator[], totalDimension)
//   Tensor<T>     include/Core/Tensor.h:12-203 (column-major, operator()(i), (i, n), [i])
//   Node / Tree   include/TreeShape/Node.h, include/TreeShape/Tree.h
//                 (bottom-up address order, isToplayer, isBottomlayer, childIdx, getLeaf)
//   Leaf          include/TreeShape/Leaf.h (dim, mode, interface)
//   LeafOperator  include/TreeOperators/LeafOperator.h (apply(grid, hA, A))
//   MLO / SOP     include/TreeOperators/MultiLeafOperator.h:11-196,
//                 include/TreeOperators/SumOfProductsOperator.h:5-135
// Test infrastructure only: the stand-ins hold what a small input file
// provides and nothing else.
#pragma once

#include <complex>
#include <cstddef>
#include <initializer_list>
#include <memory>
#include <vector>

typedef std::complex<double> cd;

class TensorShape {
 public:
  TensorShape() = default;
  TensorShape(std::initializer_list<size_t> d) : dims_(d) {}
  explicit TensorShape(std::vector<size_t> d) : dims_(std::move(d)) {}
  size_t order() const { return dims_.size(); }
  size_t operator[](size_t k) const { return dims_[k]; }
  size_t totalDimension() const {
    size_t n = 1;
    for (size_t d : dims_) n *= d;
    return n;
  }
  size_t lastBefore() const { return totalDimension() / dims_.back(); }

 private:
  std::vector<size_t> dims_;
};

template <typename T>
class Tensor {
 public:
  Tensor() = default;
  Tensor(std::initializer_list<size_t> d) : shape_(d), c_(shape_.totalDimension(), T(0)) {}
  explicit Tensor(const TensorShape& s) : shape_(s), c_(s.totalDimension(), T(0)) {}
  const TensorShape& shape() const { return shape_; }
  T& operator()(size_t i) { return c_[i]; }
  const T& operator()(size_t i) const { return c_[i]; }
  T& operator()(size_t i, size_t n) { return c_[i + shape_.lastBefore() * n]; }
  const T& operator()(size_t i, size_t n) const { return c_[i + shape_.lastBefore() * n]; }
  T& operator[](size_t i) { return c_[i]; }
  const T& operator[](size_t i) const { return c_[i]; }

 private:
  TensorShape shape_;
  std::vector<T> c_;
};
typedef Tensor<cd> Tensorcd;

class LeafInterface {};

class Leaf {
 public:
  Leaf(size_t dim, size_t mode) : dim_(dim), mode_(mode) {}
  size_t dim() const { return dim_; }
  size_t mode() const { return mode_; }
  const LeafInterface& interface() const { return grid_; }

 private:
  size_t dim_, mode_;
  LeafInterface grid_;
};

class Node {
 public:
  Node(size_t address, TensorShape shape, int parent, int child_idx, int leaf)
      : address_(address), shape_(std::move(shape)), parent_(parent), child_idx_(child_idx), leaf_(leaf) {}
  size_t address() const { return address_; }
  const TensorShape& shape() const { return shape_; }
  bool isToplayer() const { return parent_ < 0; }
  bool isBottomlayer() const { return leaf_ >= 0; }
  size_t childIdx() const { return (size_t)child_idx_; }
  const Node& parent() const { return (*nodes_)[(size_t)parent_]; }
  const Leaf& getLeaf() const { return (*leaves_)[(size_t)leaf_]; }

 private:
  friend class Tree;
  size_t address_;
  TensorShape shape_;
  int parent_, child_idx_, leaf_;
  const std::vector<Node>* nodes_ = nullptr;
  const std::vector<Leaf>* leaves_ = nullptr;
};

class Tree {
 public:
  Tree(std::vector<Node> nodes, std::vector<Leaf> leaves) : nodes_(std::move(nodes)), leaves_(std::move(leaves)) {
    for (Node& n : nodes_) {
      n.nodes_ = &nodes_;
      n.leaves_ = &leaves_;
    }
  }
  std::vector<Node>::const_iterator begin() const { return nodes_.begin(); }
  std::vector<Node>::const_iterator end() const { return nodes_.end(); }
  size_t nNodes() const { return nodes_.size(); }
  const Leaf& getLeaf(size_t mode) const { return leaves_[mode]; }

 private:
  std::vector<Node> nodes_;
  std::vector<Leaf> leaves_;
};

// A leaf operator given by its matrix (dense, column-major) or its diagonal.
class LeafOperatorcd {
 public:
  LeafOperatorcd(size_t p, bool diag, std::vector<cd> m) : p_(p), diag_(diag), m_(std::move(m)) {}
  // hA = h A on the leaf index (the first one) of a (p, n) tensor
  void apply(const LeafInterface&, Tensorcd& hA, const Tensorcd& A) const {
    const size_t n = A.shape().totalDimension() / p_;
    for (size_t c = 0; c < n; ++c)
      for (size_t i = 0; i < p_; ++i) {
        cd s = 0;
        if (diag_)
          s = m_[i] * A(i + p_ * c);
        else
          for (size_t a = 0; a < p_; ++a) s += m_[i + p_ * a] * A(a + p_ * c);
        hA(i + p_ * c) = s;
      }
  }

 private:
  size_t p_;
  bool diag_;
  std::vector<cd> m_;
};

class MLOcd {
 public:
  void push_back(std::shared_ptr<LeafOperatorcd> h, size_t mode) {
    ops_.push_back(std::move(h));
    modes_.push_back(mode);
  }
  size_t size() const { return ops_.size(); }
  const std::shared_ptr<LeafOperatorcd>& operator[](size_t k) const { return ops_[k]; }
  const std::vector<size_t>& targetLeaves() const { return modes_; }

 private:
  std::vector<std::shared_ptr<LeafOperatorcd>> ops_;
  std::vector<size_t> modes_;
};

class Hamiltonian {
 public:
  void push_back(const MLOcd& M, cd c) {
    mpos_.push_back(M);
    coeff_.push_back(c);
  }
  size_t size() const { return mpos_.size(); }
  const MLOcd& operator[](size_t l) const { return mpos_[l]; }
  cd coeff(size_t l) const { return coeff_[l]; }

 private:
  std::vector<MLOcd> mpos_;
  std::vector<cd> coeff_;
};

// TensorTreecd indexed by node
class Wavefunction {
 public:
  explicit Wavefunction(const Tree& tree) {
    for (const Node& n : tree) t_.emplace_back(n.shape());
  }
  Tensorcd& operator[](const Node& n) { return t_[n.address()]; }
  const Tensorcd& operator[](const Node& n) const { return t_[n.address()]; }

 private:
  std::vector<Tensorcd> t_;
};
