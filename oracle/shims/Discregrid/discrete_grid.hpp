// Test infrastructure: a compile-only stand-in for Discregrid (pinned commit
// ddf20dc0, CMake/SetUpExternalProjects.cmake:13-17 of the reference), which is not
// in the reference tree.  The reference's DFSPH step with Akinci2012 particle
// boundaries never evaluates a grid; these declarations follow the call sites in
// SPlisHSPlasH/TimeStep.cpp:200-420 and SPlisHSPlasH/Utilities/SDFFunctions.cpp so
// that the hot-path sources compile.  Any call aborts.
#pragma once

#include <Eigen/Dense>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <functional>

namespace Discregrid
{
	[[noreturn]] inline void not_available(const char *what)
	{
		std::fprintf(stderr, "Discregrid stand-in: %s is not available in the oracle pin build\n", what);
		std::abort();
	}

	class DiscreteGrid
	{
	public:
		using CoefficientVector = Eigen::Matrix<double, 32, 1>;
		using ContinuousFunction = std::function<double(Eigen::Vector3d const &)>;
		using MultiIndex = std::array<unsigned int, 3>;
		using Predicate = std::function<bool(Eigen::Vector3d const &, double)>;
		using SamplePredicate = std::function<bool(Eigen::Vector3d const &)>;

		DiscreteGrid() {}
		DiscreteGrid(Eigen::AlignedBox3d const &, std::array<unsigned int, 3> const &) {}
		virtual ~DiscreteGrid() {}

		virtual double interpolate(unsigned int, Eigen::Vector3d const &, Eigen::Vector3d * = nullptr) const
		{
			not_available("DiscreteGrid::interpolate");
		}
		virtual bool determineShapeFunctions(unsigned int, Eigen::Vector3d const &, std::array<unsigned int, 32> &,
			Eigen::Vector3d &, Eigen::Matrix<double, 32, 1> &, Eigen::Matrix<double, 32, 3> * = nullptr) const
		{
			not_available("DiscreteGrid::determineShapeFunctions");
		}
		virtual double interpolate(unsigned int, Eigen::Vector3d const &, const std::array<unsigned int, 32> &,
			const Eigen::Vector3d &, const Eigen::Matrix<double, 32, 1> &, Eigen::Vector3d * = nullptr,
			Eigen::Matrix<double, 32, 3> * = nullptr) const
		{
			not_available("DiscreteGrid::interpolate");
		}
		virtual unsigned int addFunction(ContinuousFunction const &, bool = false, SamplePredicate const & = nullptr)
		{
			not_available("DiscreteGrid::addFunction");
		}
		virtual void reduceField(unsigned int, Predicate) { not_available("DiscreteGrid::reduceField"); }
		void save(std::string const &) const { not_available("DiscreteGrid::save"); }
		void load(std::string const &) { not_available("DiscreteGrid::load"); }
	};

	class CubicLagrangeDiscreteGrid : public DiscreteGrid
	{
	public:
		CubicLagrangeDiscreteGrid(std::string const &) { not_available("CubicLagrangeDiscreteGrid(file)"); }
		CubicLagrangeDiscreteGrid(Eigen::AlignedBox3d const &domain, std::array<unsigned int, 3> const &res)
			: DiscreteGrid(domain, res) {}
	};

	class TriangleMesh
	{
	public:
		TriangleMesh(double const *, unsigned int const *, std::size_t, std::size_t) {}
		TriangleMesh(float const *, unsigned int const *, std::size_t, std::size_t) {}
	};

	class TriangleMeshDistance
	{
	public:
		explicit TriangleMeshDistance(TriangleMesh const &) {}
		double signedDistance(Eigen::Vector3d const &) const { not_available("TriangleMeshDistance"); }
		double signedDistanceCached(Eigen::Vector3d const &) const { not_available("TriangleMeshDistance"); }
	};
}
