// Test infrastructure: the subset of GenericParameters (pinned commit a4e2744e,
// CMake/SetUpExternalProjects.cmake:32-36 of the reference) that the reference's
// hot-path sources call, written from those call sites (e.g.
// SPlisHSPlasH/Simulation.cpp:163-278, DFSPH/TimeStepDFSPH.cpp:73-114,
// FluidModel.cpp:100-190, Viscosity/Viscosity_Weiler2018.cpp:44-74,
// pySPlisHSPlasH/ParameterObjectModule.cpp:19-32).  The library itself is not in
// the reference tree; this header only stores and forwards values so that the
// reference's own DFSPH step can be compiled and run as the oracle pin.
#pragma once

#include <functional>
#include <string>
#include <vector>
#include <stdexcept>

namespace GenParam
{
	class ParameterBase
	{
	public:
		enum DataTypes { BOOL = 0, FLOAT, DOUBLE, INT8, INT16, INT32, UINT8, UINT16, UINT32, VEC_FLOAT, VEC_DOUBLE,
			VEC_UINT8, VEC_UINT16, VEC_UINT32, VEC_INT8, VEC_INT16, VEC_INT32, ENUM, STRING, FUNCTION, NUMBER_OF_TYPES };

		template <typename T> using GetFunc = std::function<T()>;
		template <typename T> using SetFunc = std::function<void(T)>;
		template <typename T> using GetVecFunc = std::function<T *()>;
		template <typename T> using SetVecFunc = std::function<void(T *)>;

		ParameterBase(const std::string &name, const std::string &label, int type)
			: m_name(name), m_label(label), m_type(type) {}
		virtual ~ParameterBase() {}

		const std::string &getName() const { return m_name; }
		const std::string &getLabel() const { return m_label; }
		const std::string &getGroup() const { return m_group; }
		void setGroup(const std::string &g) { m_group = g; }
		const std::string &getDescription() const { return m_description; }
		void setDescription(const std::string &d) { m_description = d; }
		const std::string &getHotKey() const { return m_hotKey; }
		void setHotKey(const std::string &k) { m_hotKey = k; }
		bool getReadOnly() const { return m_readOnly; }
		void setReadOnly(bool v) { m_readOnly = v; }
		int getType() const { return m_type; }

	protected:
		std::string m_name, m_label, m_group, m_description, m_hotKey;
		int m_type;
		bool m_readOnly = false;
	};

	template <typename T> struct TypeOf;
	template <> struct TypeOf<bool> { static constexpr int value = ParameterBase::BOOL; };
	template <> struct TypeOf<float> { static constexpr int value = ParameterBase::FLOAT; };
	template <> struct TypeOf<double> { static constexpr int value = ParameterBase::DOUBLE; };
	template <> struct TypeOf<char> { static constexpr int value = ParameterBase::INT8; };
	template <> struct TypeOf<short> { static constexpr int value = ParameterBase::INT16; };
	template <> struct TypeOf<int> { static constexpr int value = ParameterBase::INT32; };
	template <> struct TypeOf<unsigned char> { static constexpr int value = ParameterBase::UINT8; };
	template <> struct TypeOf<unsigned short> { static constexpr int value = ParameterBase::UINT16; };
	template <> struct TypeOf<unsigned int> { static constexpr int value = ParameterBase::UINT32; };
	template <> struct TypeOf<std::string> { static constexpr int value = ParameterBase::STRING; };

	/** A scalar value held either through a pointer to the owner's member or through
	 *  the owner's getter/setter pair. */
	template <typename T>
	class Parameter : public ParameterBase
	{
	public:
		Parameter(const std::string &name, const std::string &label, int type, T *valuePtr)
			: ParameterBase(name, label, type), m_ptr(valuePtr) {}
		Parameter(const std::string &name, const std::string &label, int type, GetFunc<T> get, SetFunc<T> set)
			: ParameterBase(name, label, type), m_ptr(nullptr), m_get(get), m_set(set) {}
		virtual T getValue() const { return m_ptr ? *m_ptr : m_get(); }
		virtual void setValue(const T v)
		{
			if (m_ptr) *m_ptr = v;
			else if (m_set) m_set(v);
		}

	protected:
		T *m_ptr;
		GetFunc<T> m_get;
		SetFunc<T> m_set;
	};

	template <typename T>
	class NumericParameter : public Parameter<T>
	{
	public:
		NumericParameter(const std::string &name, const std::string &label, T *valuePtr)
			: Parameter<T>(name, label, TypeOf<T>::value, valuePtr) {}
		NumericParameter(const std::string &name, const std::string &label, ParameterBase::GetFunc<T> g,
			ParameterBase::SetFunc<T> s)
			: Parameter<T>(name, label, TypeOf<T>::value, g, s) {}
		void setMinValue(const T v) { m_min = v; m_hasMin = true; }
		void setMaxValue(const T v) { m_max = v; m_hasMax = true; }
		T getMinValue() const { return m_min; }
		T getMaxValue() const { return m_max; }
		void setValue(const T v) override
		{
			T w = v;
			if (m_hasMin && w < m_min) w = m_min;
			if (m_hasMax && w > m_max) w = m_max;
			Parameter<T>::setValue(w);
		}

	private:
		T m_min{}, m_max{};
		bool m_hasMin = false, m_hasMax = false;
	};

	using FloatParameter = NumericParameter<float>;
	using DoubleParameter = NumericParameter<double>;
	using IntParameter = NumericParameter<int>;
	using UnsignedIntParameter = NumericParameter<unsigned int>;

	class BoolParameter : public Parameter<bool>
	{
	public:
		BoolParameter(const std::string &name, const std::string &label, bool *valuePtr)
			: Parameter<bool>(name, label, ParameterBase::BOOL, valuePtr) {}
		BoolParameter(const std::string &name, const std::string &label, GetFunc<bool> g, SetFunc<bool> s)
			: Parameter<bool>(name, label, ParameterBase::BOOL, g, s) {}
	};

	class StringParameter : public Parameter<std::string>
	{
	public:
		StringParameter(const std::string &name, const std::string &label, std::string *valuePtr)
			: Parameter<std::string>(name, label, ParameterBase::STRING, valuePtr) {}
		StringParameter(const std::string &name, const std::string &label, GetFunc<std::string> g,
			SetFunc<std::string> s)
			: Parameter<std::string>(name, label, ParameterBase::STRING, g, s) {}
	};

	/** Enum values are numbered in the order they are added; the id variable passed in
	 *  receives that number. */
	class EnumParameter : public Parameter<int>
	{
	public:
		struct EnumValue { std::string name; int id; };
		EnumParameter(const std::string &name, const std::string &label, int *valuePtr)
			: Parameter<int>(name, label, ParameterBase::ENUM, valuePtr) {}
		EnumParameter(const std::string &name, const std::string &label, GetFunc<int> g, SetFunc<int> s)
			: Parameter<int>(name, label, ParameterBase::ENUM, g, s) {}
		void addEnumValue(const std::string &name, int &id)
		{
			id = static_cast<int>(m_values.size());
			m_values.push_back({name, id});
		}
		const std::vector<EnumValue> &getEnumValues() const { return m_values; }
		void clearEnumValues() { m_values.clear(); }

	private:
		std::vector<EnumValue> m_values;
	};

	template <typename T>
	class VectorParameter : public ParameterBase
	{
	public:
		VectorParameter(const std::string &name, const std::string &label, int type, unsigned int dim, T *valuePtr)
			: ParameterBase(name, label, type), m_dim(dim), m_ptr(valuePtr) {}
		VectorParameter(const std::string &name, const std::string &label, int type, unsigned int dim,
			GetVecFunc<T> g, SetVecFunc<T> s)
			: ParameterBase(name, label, type), m_dim(dim), m_ptr(nullptr), m_get(g), m_set(s) {}
		unsigned int getDim() const { return m_dim; }
		T *getValue() { return m_ptr ? m_ptr : m_get(); }
		void setValue(T *v)
		{
			if (m_ptr) { for (unsigned int i = 0; i < m_dim; i++) m_ptr[i] = v[i]; }
			else if (m_set) m_set(v);
		}

	private:
		unsigned int m_dim;
		T *m_ptr;
		GetVecFunc<T> m_get;
		SetVecFunc<T> m_set;
	};

	using FloatVectorParameter = VectorParameter<float>;
	using DoubleVectorParameter = VectorParameter<double>;

	template <typename T> struct VecTypeOf;
	template <> struct VecTypeOf<float> { static constexpr int value = ParameterBase::VEC_FLOAT; };
	template <> struct VecTypeOf<double> { static constexpr int value = ParameterBase::VEC_DOUBLE; };
	template <> struct VecTypeOf<unsigned int> { static constexpr int value = ParameterBase::VEC_UINT32; };
	template <> struct VecTypeOf<int> { static constexpr int value = ParameterBase::VEC_INT32; };

	class FunctionParameter : public ParameterBase
	{
	public:
		FunctionParameter(const std::string &name, const std::string &label, std::function<void()> f)
			: ParameterBase(name, label, ParameterBase::FUNCTION), m_function(f) {}
		std::function<void()> &getFunction() { return m_function; }

	private:
		std::function<void()> m_function;
	};

	/** Owner of a list of parameters addressed by the integer ids that create*()
	 *  returns, in creation order. */
	class ParameterObject
	{
	public:
		ParameterObject() {}
		virtual ~ParameterObject()
		{
			for (ParameterBase *p : m_parameters) delete p;
		}
		virtual void initParameters() {}

		unsigned int numParameters() const { return static_cast<unsigned int>(m_parameters.size()); }
		ParameterBase *getParameter(const unsigned int id) { return m_parameters[id]; }
		ParameterBase *getParameter(const std::string &name)
		{
			for (ParameterBase *p : m_parameters)
				if (p->getName() == name) return p;
			return nullptr;
		}
		int getParameterIndex(const std::string &name)
		{
			for (unsigned int i = 0; i < m_parameters.size(); i++)
				if (m_parameters[i]->getName() == name) return static_cast<int>(i);
			return -1;
		}
		void setGroup(const unsigned int id, const std::string &g) { m_parameters[id]->setGroup(g); }
		void setDescription(const unsigned int id, const std::string &d) { m_parameters[id]->setDescription(d); }
		void setHotKey(const unsigned int id, const std::string &k) { m_parameters[id]->setHotKey(k); }

		template <typename T>
		int createNumericParameter(const std::string &name, const std::string &label, T *valuePtr)
		{
			return add(new NumericParameter<T>(name, label, valuePtr));
		}
		template <typename T>
		int createNumericParameter(const std::string &name, const std::string &label,
			ParameterBase::GetFunc<T> g, ParameterBase::SetFunc<T> s = nullptr)
		{
			return add(new NumericParameter<T>(name, label, g, s));
		}
		int createBoolParameter(const std::string &name, const std::string &label, bool *valuePtr)
		{
			return add(new BoolParameter(name, label, valuePtr));
		}
		int createBoolParameter(const std::string &name, const std::string &label, ParameterBase::GetFunc<bool> g,
			ParameterBase::SetFunc<bool> s = nullptr)
		{
			return add(new BoolParameter(name, label, g, s));
		}
		int createEnumParameter(const std::string &name, const std::string &label, int *valuePtr)
		{
			return add(new EnumParameter(name, label, valuePtr));
		}
		int createEnumParameter(const std::string &name, const std::string &label, ParameterBase::GetFunc<int> g,
			ParameterBase::SetFunc<int> s = nullptr)
		{
			return add(new EnumParameter(name, label, g, s));
		}
		int createStringParameter(const std::string &name, const std::string &label, std::string *valuePtr)
		{
			return add(new StringParameter(name, label, valuePtr));
		}
		int createStringParameter(const std::string &name, const std::string &label,
			ParameterBase::GetFunc<std::string> g, ParameterBase::SetFunc<std::string> s)
		{
			return add(new StringParameter(name, label, g, s));
		}
		template <typename T>
		int createVectorParameter(const std::string &name, const std::string &label, const unsigned int dim, T *valuePtr)
		{
			return add(new VectorParameter<T>(name, label, VecTypeOf<T>::value, dim, valuePtr));
		}
		template <typename T>
		int createVectorParameter(const std::string &name, const std::string &label, const unsigned int dim,
			ParameterBase::GetVecFunc<T> g, ParameterBase::SetVecFunc<T> s)
		{
			return add(new VectorParameter<T>(name, label, VecTypeOf<T>::value, dim, g, s));
		}
		int createFunctionParameter(const std::string &name, const std::string &label, std::function<void()> f)
		{
			return add(new FunctionParameter(name, label, f));
		}

		template <typename T>
		T getValue(const unsigned int id)
		{
			return static_cast<Parameter<T> *>(m_parameters[id])->getValue();
		}
		template <typename T>
		void setValue(const unsigned int id, const T v)
		{
			ParameterBase *p = m_parameters[id];
			switch (p->getType())
			{
			case ParameterBase::BOOL: static_cast<Parameter<bool> *>(p)->setValue(static_cast<bool>(v)); break;
			case ParameterBase::FLOAT: static_cast<NumericParameter<float> *>(p)->setValue(static_cast<float>(v)); break;
			case ParameterBase::DOUBLE: static_cast<NumericParameter<double> *>(p)->setValue(static_cast<double>(v)); break;
			case ParameterBase::INT32: static_cast<NumericParameter<int> *>(p)->setValue(static_cast<int>(v)); break;
			case ParameterBase::UINT32:
				static_cast<NumericParameter<unsigned int> *>(p)->setValue(static_cast<unsigned int>(v));
				break;
			case ParameterBase::ENUM: static_cast<Parameter<int> *>(p)->setValue(static_cast<int>(v)); break;
			default: throw std::runtime_error("ParameterObject::setValue: unsupported type for " + p->getName());
			}
		}
		void setValue(const unsigned int id, const std::string &v)
		{
			static_cast<Parameter<std::string> *>(m_parameters[id])->setValue(v);
		}
		template <typename T>
		T *getVecValue(const unsigned int id)
		{
			return static_cast<VectorParameter<T> *>(m_parameters[id])->getValue();
		}
		template <typename T>
		void setVecValue(const unsigned int id, T *v)
		{
			static_cast<VectorParameter<T> *>(m_parameters[id])->setValue(v);
		}

	protected:
		int add(ParameterBase *p)
		{
			m_parameters.push_back(p);
			return static_cast<int>(m_parameters.size()) - 1;
		}
		std::vector<ParameterBase *> m_parameters;
	};
}
