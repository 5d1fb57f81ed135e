// Test infrastructure: a stand-in for CompactNSearch (pinned commit a9ab7c71,
// CMake/NeighborhoodSearch.cmake:32-36 of the reference), which is not in the
// reference tree.  It implements the interface the reference calls
// (SPlisHSPlasH/NeighborhoodSearch.h:12, Simulation.cpp:145-151,606-642,696-756,
// Simulation.h:451-473, FluidModel.cpp:214-216,323,336-346,
// BoundaryModel_Akinci2012.cpp:52-67,108-126, SimulationDataDFSPH.cpp:83-101) with
// this project's documented neighbour predicate, so that the reference's own
// DFSPH step can be compiled and run as the oracle pin:
//   * j is a neighbour of i when |x_i - x_j|^2 < r^2, the squared distance formed in
//     the build's Real as ((dx*dx + dy*dy) + dz*dz), a point never its own neighbour;
//   * each list is in ascending index order (CompactNSearch's own order is
//     unpinned; sums over a list are order-dependent only at rounding level);
//   * z_sort() keeps the identity order, so sort_field() leaves fields unchanged
//     (the reference compares runs by particle id, never by index).
// Activation: active(i, j) means "point set i searches neighbours in point set j".
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace CompactNSearch
{
#ifdef USE_DOUBLE
	using Real = double;
#else
	using Real = float;
#endif

	class NeighborhoodSearch;

	class PointSet
	{
	public:
		PointSet(Real const *x, std::size_t n, bool dynamic, void *user_data)
			: m_x(x), m_n(n), m_dynamic(dynamic), m_user_data(user_data) {}

		std::size_t n_points() const { return m_n; }
		std::size_t n_neighbors(unsigned int point_set, unsigned int i) const
		{
			return point_set < m_neighbors.size() && i < m_neighbors[point_set].size()
				? m_neighbors[point_set][i].size() : 0;
		}
		unsigned int neighbor(unsigned int point_set, unsigned int i, unsigned int k) const
		{
			return m_neighbors[point_set][i][k];
		}
		std::vector<unsigned int> const &neighbor_list(unsigned int point_set, unsigned int i) const
		{
			return m_neighbors[point_set][i];
		}
		void *get_user_data() const { return m_user_data; }
		bool is_dynamic() const { return m_dynamic; }
		void set_dynamic(bool v) { m_dynamic = v; }
		Real const *GetPoints() const { return m_x; }
		Real const *point(unsigned int i) const { return m_x + 3 * static_cast<std::size_t>(i); }

		/** z_sort() keeps the identity permutation, so sorting a field is a no-op. */
		template <typename T> void sort_field(T *) const {}
		unsigned int get_sort_table_entry(unsigned int i) const { return i; }

	private:
		friend class NeighborhoodSearch;
		Real const *m_x;
		std::size_t m_n;
		bool m_dynamic;
		void *m_user_data;
		// m_neighbors[other point set][point] = ascending neighbour indices
		std::vector<std::vector<std::vector<unsigned int>>> m_neighbors;
	};

	class NeighborhoodSearch
	{
	public:
		NeighborhoodSearch(Real r, bool /*erase_empty_cells*/ = false) : m_r(r) {}

		void set_radius(Real r) { m_r = r; }
		Real radius() const { return m_r; }

		unsigned int add_point_set(Real const *x, std::size_t n, bool is_dynamic = true,
			bool search_neighbors = true, bool find_neighbors = true, void *user_data = nullptr)
		{
			m_sets.emplace_back(x, n, is_dynamic, user_data);
			m_search.push_back(search_neighbors);
			m_find.push_back(find_neighbors);
			const std::size_t k = m_sets.size();
			std::vector<std::vector<char>> t(k, std::vector<char>(k, 0));
			for (std::size_t i = 0; i + 1 < k; i++)
				for (std::size_t j = 0; j + 1 < k; j++)
					t[i][j] = m_active[i][j];
			for (std::size_t j = 0; j < k; j++)
			{
				t[k - 1][j] = m_search[k - 1] && m_find[j];
				t[j][k - 1] = m_search[j] && m_find[k - 1];
			}
			m_active.swap(t);
			return static_cast<unsigned int>(k - 1);
		}

		void resize_point_set(unsigned int i, Real const *x, std::size_t n)
		{
			m_sets[i].m_x = x;
			m_sets[i].m_n = n;
		}

		PointSet const &point_set(unsigned int i) const { return m_sets[i]; }
		PointSet &point_set(unsigned int i) { return m_sets[i]; }
		std::size_t n_point_sets() const { return m_sets.size(); }
		std::vector<PointSet> const &point_sets() const { return m_sets; }

		void set_active(bool active)
		{
			for (auto &row : m_active) std::fill(row.begin(), row.end(), static_cast<char>(active));
		}
		void set_active(unsigned int i, unsigned int j, bool active) { m_active[i][j] = active; }
		void set_active(unsigned int i, bool search_neighbors = true, bool find_neighbors = true)
		{
			for (std::size_t j = 0; j < m_sets.size(); j++)
			{
				m_active[i][j] = search_neighbors;
				m_active[j][i] = find_neighbors;
			}
			m_active[i][i] = search_neighbors && find_neighbors;
		}
		bool is_active(unsigned int i, unsigned int j) const { return m_active[i][j] != 0; }

		void update_point_sets() {}
		void update_activation_table() {}
		void z_sort() {}

		/** Neighbour lists of every active pair (i searches in j), from scratch. */
		void find_neighbors(bool /*points_changed*/ = true)
		{
			const std::size_t ns = m_sets.size();
			for (std::size_t i = 0; i < ns; i++)
			{
				m_sets[i].m_neighbors.resize(ns);
				for (std::size_t j = 0; j < ns; j++)
					if (m_active[i][j]) search_pair(i, j);
			}
		}

	private:
		struct Grid
		{
			long long lo[3] = {0, 0, 0};
			long long dim[3] = {0, 0, 0};
			std::vector<unsigned int> start; // size cells + 1
			std::vector<unsigned int> idx;   // point indices grouped by cell, ascending within a cell
		};

		Real cell_size() const { return m_r * static_cast<Real>(1.0001); }

		long long cell_coord(Real v) const { return static_cast<long long>(std::floor(v / cell_size())); }

		void build_grid(PointSet const &s, Grid &g) const
		{
			const std::size_t n = s.m_n;
			g.start.clear();
			g.idx.clear();
			if (n == 0) return;
			long long lo[3], hi[3];
			for (int d = 0; d < 3; d++) { lo[d] = cell_coord(s.m_x[d]); hi[d] = lo[d]; }
			for (std::size_t p = 0; p < n; p++)
				for (int d = 0; d < 3; d++)
				{
					const long long c = cell_coord(s.m_x[3 * p + d]);
					lo[d] = std::min(lo[d], c);
					hi[d] = std::max(hi[d], c);
				}
			long long cells = 1;
			for (int d = 0; d < 3; d++)
			{
				g.lo[d] = lo[d];
				g.dim[d] = hi[d] - lo[d] + 1;
				cells *= g.dim[d];
			}
			if (cells > (1ll << 28))
			{
				std::fprintf(stderr, "CompactNSearch stand-in: point set spans %lld cells\n", cells);
				std::abort();
			}
			std::vector<unsigned int> cid(n);
			g.start.assign(static_cast<std::size_t>(cells) + 1, 0);
			for (std::size_t p = 0; p < n; p++)
			{
				long long c[3];
				for (int d = 0; d < 3; d++) c[d] = cell_coord(s.m_x[3 * p + d]) - g.lo[d];
				cid[p] = static_cast<unsigned int>((c[2] * g.dim[1] + c[1]) * g.dim[0] + c[0]);
				g.start[cid[p] + 1]++;
			}
			for (long long c = 0; c < cells; c++) g.start[c + 1] += g.start[c];
			g.idx.resize(n);
			std::vector<unsigned int> fill(g.start.begin(), g.start.end() - 1);
			for (std::size_t p = 0; p < n; p++) g.idx[fill[cid[p]]++] = static_cast<unsigned int>(p);
		}

		void search_pair(std::size_t i, std::size_t j)
		{
			PointSet &a = m_sets[i];
			PointSet const &b = m_sets[j];
			Grid g;
			build_grid(b, g);
			auto &lists = a.m_neighbors[j];
			lists.assign(a.m_n, std::vector<unsigned int>());
			if (b.m_n == 0) return;
			const Real r2 = m_r * m_r;
			const bool same = (i == j);
#pragma omp parallel for schedule(dynamic, 256)
			for (long long p = 0; p < static_cast<long long>(a.m_n); p++)
			{
				const Real *xp = a.m_x + 3 * p;
				long long c[3];
				for (int d = 0; d < 3; d++) c[d] = cell_coord(xp[d]) - g.lo[d];
				std::vector<unsigned int> &out = lists[p];
				for (long long dz = -1; dz <= 1; dz++)
				{
					const long long z = c[2] + dz;
					if (z < 0 || z >= g.dim[2]) continue;
					for (long long dy = -1; dy <= 1; dy++)
					{
						const long long y = c[1] + dy;
						if (y < 0 || y >= g.dim[1]) continue;
						for (long long dx = -1; dx <= 1; dx++)
						{
							const long long x = c[0] + dx;
							if (x < 0 || x >= g.dim[0]) continue;
							const long long cell = (z * g.dim[1] + y) * g.dim[0] + x;
							for (unsigned int k = g.start[cell]; k < g.start[cell + 1]; k++)
							{
								const unsigned int q = g.idx[k];
								if (same && q == static_cast<unsigned int>(p)) continue;
								const Real *xq = b.m_x + 3 * static_cast<std::size_t>(q);
								const Real ex = xp[0] - xq[0];
								const Real ey = xp[1] - xq[1];
								const Real ez = xp[2] - xq[2];
								const Real exx = ex * ex;
								const Real eyy = ey * ey;
								const Real ezz = ez * ez;
								const Real d2 = (exx + eyy) + ezz;
								if (d2 < r2) out.push_back(q);
							}
						}
					}
				}
				std::sort(out.begin(), out.end());
			}
		}

		Real m_r;
		std::vector<PointSet> m_sets;
		std::vector<char> m_search, m_find;
		std::vector<std::vector<char>> m_active;
	};
}
