// Test infrastructure: the reference's particle state files, written and read through partio
// (vendored in the reference tree, extern/partio) the way the reference's simulator does it
// (SimulatorBase::writeFluidParticlesState / readFluidParticlesState,
// Simulator/SimulatorBase.cpp:2062-2192): every field of the fluid model marked storeData,
// under its name, as partio FLOAT (scalar), INT (uint) or VECTOR (3-vector) attributes; on
// reading, every attribute whose name matches a field of the model is assigned in record
// order.  Linked with the reference's objects and oracle/ref_driver.cpp, so the reference's
// Simulation set up by ref_create is the one saved and restored.
#include "SPlisHSPlasH/Simulation.h"
#include "SPlisHSPlasH/TimeManager.h"
#include "Utilities/BinaryFileReaderWriter.h"
#include "Partio.h"

#include <vector>

using namespace SPH;

extern "C" {

/** Writes fluid model 0's state file; returns the number of attributes written, or -1. */
int state_write(const char *path)
{
    FluidModel *model = Simulation::getCurrent()->getFluidModel(0);
    Partio::ParticlesDataMutable &pd = *Partio::create();
    struct Col { unsigned int field; Partio::ParticleAttribute attr; };
    std::vector<Col> cols;
    for (unsigned int j = 0; j < model->numberOfFields(); j++) {
        const FieldDescription &fd = model->getField(j);
        if (!fd.storeData) continue;
        if (fd.type == FieldType::Scalar) cols.push_back({j, pd.addAttribute(fd.name.c_str(), Partio::FLOAT, 1)});
        else if (fd.type == FieldType::UInt) cols.push_back({j, pd.addAttribute(fd.name.c_str(), Partio::INT, 1)});
        else if (fd.type == FieldType::Vector3) cols.push_back({j, pd.addAttribute(fd.name.c_str(), Partio::VECTOR, 3)});
    }
    for (unsigned int i = 0; i < model->numActiveParticles(); i++) {
        const Partio::ParticleIndex p = pd.addParticle();
        for (const Col &c : cols) {
            const FieldDescription &fd = model->getField(c.field);
            if (fd.type == FieldType::UInt) {
                *pd.dataWrite<int>(c.attr, p) = (int)*static_cast<unsigned int *>(fd.getFct(i));
            } else {
                float *dst = pd.dataWrite<float>(c.attr, p);
                const Real *src = static_cast<Real *>(fd.getFct(i));
                for (int k = 0; k < c.attr.count; k++) dst[k] = (float)src[k];
            }
        }
    }
    Partio::write(path, pd, true);
    pd.release();
    return (int)cols.size();
}

/** Reads a state file into fluid model 0; returns the number of attributes matched, or -1
 *  when the file cannot be read or its point count differs from the model's. */
int state_read(const char *path)
{
    FluidModel *model = Simulation::getCurrent()->getFluidModel(0);
    Partio::ParticlesDataMutable *data = Partio::read(path);
    if (!data) return -1;
    if ((unsigned int)data->numParticles() != model->numActiveParticles()) {
        data->release();
        return -1;
    }
    int matched = 0;
    for (int a = 0; a < data->numAttributes(); a++) {
        Partio::ParticleAttribute attr;
        data->attributeInfo(a, attr);
        for (unsigned int j = 0; j < model->numberOfFields(); j++) {
            const FieldDescription &fd = model->getField(j);
            if (fd.name != attr.name) continue;
            matched++;
            for (int i = 0; i < data->numParticles(); i++) {
                if (fd.type == FieldType::UInt) {
                    *static_cast<unsigned int *>(fd.getFct(i)) = (unsigned int)data->data<int>(attr, i)[0];
                } else if (fd.type == FieldType::Scalar) {
                    *static_cast<Real *>(fd.getFct(i)) = data->data<float>(attr, i)[0];
                } else if (fd.type == FieldType::Vector3) {
                    const float *v = data->data<float>(attr, i);
                    Real *dst = static_cast<Real *>(fd.getFct(i));
                    for (int k = 0; k < 3; k++) dst[k] = v[k];
                }
            }
        }
    }
    data->release();
    return matched;
}

/** The library's section of the simulator's .bin state file, written as SimulatorBase::saveState
 *  writes it (Simulator/SimulatorBase.cpp:1724-1725): TimeManager::saveState, then
 *  Simulation::saveState (time, step size, W(0), the fluid models' particle states and emitter
 *  counts, the boundary models' sort flags and point-set indices, the time step's own state);
 *  returns 0, or -1 when the file cannot be opened. */
int sim_state_write(const char *path)
{
    BinaryFileWriter w;
    if (!w.openFile(path)) return -1;
    TimeManager::getCurrent()->saveState(w);
    Simulation::getCurrent()->saveState(w);
    w.closeFile();
    return 0;
}

/** Reads that section back as SimulatorBase::loadState does (:1805-1806); the particle files
 *  follow with state_read, in that order. */
int sim_state_read(const char *path)
{
    BinaryFileReader r;
    if (!r.openFile(path)) return -1;
    TimeManager::getCurrent()->loadState(r);
    Simulation::getCurrent()->loadState(r);
    r.closeFile();
    return 0;
}

/** Attribute names of a BGEO file, separated by '\n', with their partio types (F, I or V)
 *  and point count; for checking a file's layout with partio itself. */
int bgeo_describe(const char *path, char *out, int cap, int *npoints)
{
    Partio::ParticlesData *data = Partio::read(path);
    if (!data) return -1;
    std::string s;
    for (int a = 0; a < data->numAttributes(); a++) {
        Partio::ParticleAttribute attr;
        data->attributeInfo(a, attr);
        s += attr.name + ":" + (attr.type == Partio::FLOAT ? "F" : attr.type == Partio::INT ? "I" : "V") +
             std::to_string(attr.count) + "\n";
    }
    *npoints = data->numParticles();
    data->release();
    if ((int)s.size() + 1 > cap) return -2;
    std::copy(s.begin(), s.end(), out);
    out[s.size()] = 0;
    return (int)s.size();
}

/** All values of attribute `name` (or "position") as doubles, point by point; returns their
 *  number, or -1 when the file or the attribute is missing or out has less room. */
int bgeo_column(const char *path, const char *name, double *out, int cap)
{
    Partio::ParticlesData *data = Partio::read(path);
    if (!data) return -1;
    Partio::ParticleAttribute attr;
    int m = -1;
    if (data->attributeInfo(name, attr) && data->numParticles() * attr.count <= cap) {
        m = 0;
        for (int i = 0; i < data->numParticles(); i++)
            for (int k = 0; k < attr.count; k++)
                out[m++] = attr.type == Partio::INT ? (double)data->data<int>(attr, i)[k]
                                                    : (double)data->data<float>(attr, i)[k];
    }
    data->release();
    return m;
}

}  // extern "C"
