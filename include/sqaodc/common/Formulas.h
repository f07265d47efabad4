// Formulas.h -- the formula interfaces of the sqaod C++ API
// (sqaodc/common/Formulas.h:7-70 of the reference): QUBO and Ising energies
// and the QUBO -> Ising conversion for dense and bipartite graphs.  The method
// names, argument order and meanings are the reference's, so code written
// against it compiles unchanged.  Bits x are {0, 1} and spins q are {-1, +1},
// held in real-typed vectors and matrices as in the reference; W and J of a
// dense graph must be symmetric.
#pragma once

#include <sqaodc/common/Common.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

namespace sqaod {

template <class real>
struct DenseGraphFormulas : NullBase {
    typedef MatrixType<real> Matrix;
    typedef VectorType<real> Vector;

    virtual ~DenseGraphFormulas() {}

    // E = x W x^T of one bit vector
    virtual void calculate_E(real *E, const Matrix &W, const Vector &x) = 0;

    // E[i] = x_i W x_i^T of every row of x
    virtual void calculate_E(Vector *E, const Matrix &W, const Matrix &x) = 0;

    // h, J (zero diagonal), c with E_qubo(x) = E_ising(2 x - 1)
    virtual void calculateHamiltonian(Vector *h, Matrix *J, real *c, const Matrix &W) = 0;

    // E = -c - h q^T - q J q^T of one spin vector
    virtual void calculate_E(real *E, const Vector &h, const Matrix &J, real c, const Vector &q) = 0;

    // the same for every row of q
    virtual void calculate_E(Vector *E, const Vector &h, const Matrix &J, real c, const Matrix &q) = 0;
};

template <class real>
struct BipartiteGraphFormulas : NullBase {
    typedef MatrixType<real> Matrix;
    typedef VectorType<real> Vector;

    virtual ~BipartiteGraphFormulas() {}

    // E = b0 x0^T + b1 x1^T + x1 W x0^T (W is N1 x N0)
    virtual void calculate_E(real *E, const Vector &b0, const Vector &b1, const Matrix &W, const Vector &x0,
                             const Vector &x1) = 0;

    // the same for every pair of rows (x0_i, x1_i)
    virtual void calculate_E(Vector *E, const Vector &b0, const Vector &b1, const Matrix &W, const Matrix &x0,
                             const Matrix &x1) = 0;

    // E[i1][i0] for every combination of a row of x1 and a row of x0
    virtual void calculate_E_2d(Matrix *E, const Vector &b0, const Vector &b1, const Matrix &W, const Matrix &x0,
                                const Matrix &x1) = 0;

    virtual void calculateHamiltonian(Vector *h0, Vector *h1, Matrix *J, real *c, const Vector &b0,
                                      const Vector &b1, const Matrix &W) = 0;

    // E = -c - h0 q0^T - h1 q1^T - q1 J q0^T
    virtual void calculate_E(real *E, const Vector &h0, const Vector &h1, const Matrix &J, real c,
                             const Vector &q0, const Vector &q1) = 0;

    virtual void calculate_E(Vector *E, const Vector &h0, const Vector &h1, const Matrix &J, real c,
                             const Matrix &q0, const Matrix &q1) = 0;
};

}  // namespace sqaod

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
