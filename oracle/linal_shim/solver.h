/*
 * phelm::Solver<T> / SparseSolverAdder stand-in for the reference build
 * (project-written, test infrastructure).  add() accumulates in call order,
 * mult_vector() is a CSR product in ascending column order, solve() is the
 * oracle's GMRES (orc_csr_solve in oracle/orc_linalg.c).
 */
#ifndef ORC_SOLVER_SHIM_H
#define ORC_SOLVER_SHIM_H
#include <vector>
#include <map>
#include <cstdio>
#include "linal.h"
#include "../phelm_oracle.h"

namespace phelm {

class SparseSolverAdder {
public:
	virtual ~SparseSolverAdder() {}
	virtual void add(int i, int j, double a) = 0;
};

template <typename T>
class Solver : public SparseSolverAdder {
	int n_;
	std::vector<std::map<int, T> > rows_;
	orc_csr csr_;
	bool built_;
	void build() {
		if (built_) return;
		orc_csr_free(&csr_);
		orc_builder *b = orc_builder_new(n_, 1 << 30);
		for (int i = 0; i < n_; ++i)
			for (typename std::map<int, T>::const_iterator it = rows_[i].begin(); it != rows_[i].end(); ++it)
				orc_builder_add(b, i, it->first, (double)it->second);
		orc_builder_finish(b, &csr_);
		int mx = 0;
		for (int k = 0; k < orc_csr_nnz(&csr_); ++k) if (csr_.col[k] + 1 > mx) mx = csr_.col[k] + 1;
		csr_.m = mx > n_ ? mx : n_;
		built_ = true;
	}
public:
	typedef T data_type;
	explicit Solver(int n) : n_(n), rows_(n), built_(false) { memset(&csr_, 0, sizeof(csr_)); }
	~Solver() { orc_csr_free(&csr_); }
	void add(int i, int j, double a) { rows_[i][j] += (T)a; built_ = false; }
	void mult_vector(T *y, const T *x) {
		for (int i = 0; i < n_; ++i) {
			T s = 0;
			for (typename std::map<int, T>::const_iterator it = rows_[i].begin(); it != rows_[i].end(); ++it)
				s += it->second * x[it->first];
			y[i] = s;
		}
	}
	void solve(T *x, const T *b) {
		build();
		std::vector<double> xb(n_), bb(b, b + n_);
		orc_csr_solve(&csr_, &xb[0], &bb[0]);
		for (int i = 0; i < n_; ++i) x[i] = (T)xb[i];
	}
	/* test access: the accumulated rows */
	const std::vector<std::map<int, T> > &rows() const { return rows_; }
	int size() const { return n_; }
	void print(FILE * = stdout) {}
	void dump(FILE * = stdout) {}
};

} /* namespace phelm */
#endif
