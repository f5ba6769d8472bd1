// Stand-in for the reference's headers when type-checking the plugin
// translation unit of INTEGRATION.md: the types and members that unit uses,
// with the reference's names, argument types and enum values (grid.h:29,
// 292-304; fluidsolver.h; general.h's errMsg/debMsg).  Declarations only;
// nothing here runs.
#pragma once
#include <sstream>
#include <stdexcept>
#include <string>

#define PYTHON()

namespace Manta {
typedef float Real;
struct Vec3 {
  Real x, y, z;
};
struct Vec3i {
  int x, y, z;
};
enum Preconditioner { PcNone = 0, PcMIC = 1, PcMGDynamic = 2, PcMGStatic = 3 };

class FluidSolver {
 public:
  Vec3i getGridSize() const;
  bool is3D() const;
  Real getDt() const;
};

class GridBase {
 public:
  enum GridType { TypeNone = 0, TypeReal = 1, TypeInt = 2, TypeVec3 = 4, TypeMAC = 8, TypeLevelset = 16, TypeFlags = 32 };
  int getType() const;
  FluidSolver* getParent() const;
  int getSizeX() const;
  int getSizeY() const;
  int getSizeZ() const;
};
template <class T>
class Grid : public GridBase {
 public:
  T& get(int idx);
};
class MACGrid : public Grid<Vec3> {};
class FlagGrid : public Grid<int> {
 public:
  enum CellType { TypeNone = 0, TypeFluid = 1, TypeObstacle = 2, TypeEmpty = 4, TypeInflow = 8, TypeOutflow = 16,
                  TypeOpen = 32, TypeStick = 64 };
};
class LevelsetGrid : public Grid<Real> {};
typedef long long IndexInt;
// particle.h:182-191, 193, 276, 306
struct BasicParticleData {
  Vec3 pos;
  int flag;
};
class BasicParticleSystem {
 public:
  BasicParticleData& operator[](IndexInt idx);
  const BasicParticleData& operator[](IndexInt idx) const;
  IndexInt size() const;
  FluidSolver* getParent() const;
};
class ParticleDataBase {
 public:
  virtual ~ParticleDataBase();
};
template <class T>
class ParticleDataImpl : public ParticleDataBase {
 public:
  T& operator[](IndexInt idx);
  const T& operator[](IndexInt idx) const;
  IndexInt size() const;
};
class ParticleIndexSystem;

[[noreturn]] inline void errMsgText(const std::string& s) { throw std::runtime_error(s); }
}  // namespace Manta

#define errMsg(msg)                  \
  do {                               \
    std::ostringstream o_;           \
    o_ << msg;                       \
    Manta::errMsgText(o_.str());     \
  } while (0)
#define debMsg(msg, level)           \
  do {                               \
    std::ostringstream o_;           \
    o_ << msg;                       \
    (void)(level);                   \
  } while (0)
