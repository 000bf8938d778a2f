# ref.mk -- builds the UNMODIFIED reference engine from its own sources, where they
# lie, into oracle/_ref/ (git-ignored). Test infrastructure only: it pins the CPU
# restatement and generates golden fixtures; the product never links it.
#
#   make -f oracle/ref.mk REF=<reference source tree> -j8
#
# REF is required (command line or environment): without it, or where it holds no sources,
# nothing is built.
#
# The list is the reference's BIOSPRING_CORE_SOURCES (CMakeLists.txt:131-175) minus
# src/IO/io.cpp and src/IO/NetCDF*.cpp, which need the absent NetCDF library and are
# not on the step path, plus the xdrfile C sources (CMakeLists.txt:129). Object names
# carry their directory so that topology/Particle.cpp and spn/Particle.cpp (and the
# two PDBTrajectoryWriter.cpp) do not collide. Flags follow the reference's OpenMP
# build (-O2 -fopenmp -DOPENMP_SUPPORT, C++20). -ffp-contract=off keeps float
# arithmetic identical on x86-64 and aarch64.

REF ?=
HERE := $(dir $(lastword $(MAKEFILE_LIST)))
OUT := $(HERE)_ref
OBJ := $(OUT)/obj

CXX ?= g++
CC ?= gcc
FLAGS := -O2 -fopenmp -DOPENMP_SUPPORT -fPIC -ffp-contract=off -w
INC := -I$(OUT)/gen -I$(REF)/src -I$(REF)/src/spn -I$(REF)/src/IO/xdrfile/src

CORE := \
  src/cli/argparse.cpp \
  src/configuration/SafeConfigurationReader.cpp \
  src/forcefield/ForceField.cpp \
  src/grid/GridCoordinatesSystem.cpp \
  src/grid/PotentialGrid.cpp \
  src/reduce/ParticleGroup.cpp \
  src/reduce/Reduce.cpp \
  src/reduce/Reducer.cpp \
  src/reduce/ReduceRule.cpp \
  src/IO/CSVSampleWriter.cpp \
  src/IO/ForceFieldReader.cpp \
  src/IO/OpenDXReader.cpp \
  src/IO/PDBReader.cpp \
  src/IO/PDBTrajectoryWriter.cpp \
  src/IO/PDBWriter.cpp \
  src/IO/PQRReader.cpp \
  src/IO/PQRWriter.cpp \
  src/IO/ReduceRuleReader.cpp \
  src/IO/XTCTrajWriter.cpp \
  src/IO/modern/CSVTrajectoryWriter.cpp \
  src/IO/modern/PDBTrajectoryWriter.cpp \
  src/IO/modern/XTCTrajectoryWriter.cpp \
  src/IO/modern/TrajectoryManager.cpp \
  src/Constraint.cpp \
  src/InsertionVector.cpp \
  src/Vector3f.cpp \
  src/interactor/Interactor.cpp \
  src/logging.cpp \
  src/measure.cpp \
  src/spn/Particle.cpp \
  src/spn/ParticleProperty.cpp \
  src/spn/Spring.cpp \
  src/spn/SpringNetwork.cpp \
  src/topology/Particle.cpp \
  src/topology/ParticleCollection.cpp \
  src/topology/ParticleProperties.cpp \
  src/rigidbody/RigidBody.cpp \
  src/rigidbody/matrix.cpp \
  src/rigidbody/Quaternion.cpp \
  src/rigidbody/RigidBodiesManager.cpp

XDR := src/IO/xdrfile/src/xdrfile.c src/IO/xdrfile/src/xdrfile_trr.c src/IO/xdrfile/src/xdrfile_xtc.c

objname = $(OBJ)/$(subst /,__,$(basename $(1))).o
CORE_OBJS := $(foreach s,$(CORE),$(call objname,$(s)))
XDR_OBJS := $(foreach s,$(XDR),$(call objname,$(s)))
DRIVER_OBJ := $(OBJ)/ref_driver.o

ifeq ($(and $(REF),$(wildcard $(REF)/src/spn/SpringNetwork.cpp)),)
all:
	@echo "reference sources not present: oracle/_ref is not built"
else
all: $(OUT)/libbsref.so
endif

$(OUT)/gen/version.h: $(REF)/src/version.h.in
	@mkdir -p $(OUT)/gen
	sed 's/@BIOSPRING_VERSION@/1.1.1/' $< > $@

define CXX_RULE
$(call objname,$(1)): $(REF)/$(1) $(OUT)/gen/version.h
	@mkdir -p $(OBJ)
	$(CXX) -std=c++20 $(FLAGS) $(INC) -c $$< -o $$@
endef
$(foreach s,$(CORE),$(eval $(call CXX_RULE,$(s))))

define CC_RULE
$(call objname,$(1)): $(REF)/$(1)
	@mkdir -p $(OBJ)
	$(CC) $(FLAGS) $(INC) -c $$< -o $$@
endef
$(foreach s,$(XDR),$(eval $(call CC_RULE,$(s))))

$(DRIVER_OBJ): $(HERE)ref_driver.cpp $(HERE)../include/biospring_gb300.h $(OUT)/gen/version.h
	@mkdir -p $(OBJ)
	$(CXX) -std=c++20 $(FLAGS) $(INC) -c $< -o $@

$(OUT)/libbsref.so: $(CORE_OBJS) $(XDR_OBJS) $(DRIVER_OBJ)
	$(CXX) -shared -fopenmp -o $@ $^

clean:
	rm -rf $(OUT)

.PHONY: all clean
