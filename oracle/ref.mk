# Build recipe for the reference CPU implementation of the Tersoff + ILP path.
#
# Test infrastructure only: the binary built here is the pinned checker that the
# oracle restatement (oracle/lmff_oracle.c) and the golden fixtures under
# tests/golden/ are validated against.  Nothing in the product links it.
#
# The reference is a LAMMPS 3Mar2020 source snapshot.  Its own build system
# (Make.sh / Makefile / Install.sh) is NOT run: this short Makefile compiles the
# reference's sources where they lie and writes every output (objects, the few
# headers LAMMPS normally generates, the harness binary) under $(OUT) only.
#
#   make -f oracle/ref.mk REF=<reference checkout> -j8
#
# Sources compiled:
#   Rft/*.cpp (core, minus main.cpp; Rft/USER-MISC/pair_ilp_graphene_hbn.cpp is
#   byte-identical to Baseline's), Rft/MOLECULE/*.cpp (atom_style full),
#   Rft/MANYBODY/pair_tersoff.cpp, Rft/USER-MISC/pair_ilp_graphene_hbn.cpp,
#   Rft/STUBS/mpi.c, and three stock core files that the snapshot omits but
#   SWLMFF-5GCC/ carries (atom_vec_ellipsoid, dihedral_hybrid, improper_hybrid,
#   plus headers accelerator_kokkos.h, accelerator_omp.h, math_vector.h).
# Rft/npair_full_bin.cpp is used (LMFF/npair_full_bin.cpp returns early).

REF ?= /root/reference
OUT ?= oracle/_ref
SRC := $(REF)/Rft
EXTRA := $(REF)/SWLMFF-5GCC
GEN := $(OUT)/gen
OBJ := $(OUT)/obj

CXX ?= g++
CC ?= gcc
# -ffp-contract=off keeps the reference arithmetic identical on x86 and Arm hosts.
CXXFLAGS := -O2 -std=c++11 -w -ffp-contract=off -DLAMMPS_MEMALIGN=64 -DLAMMPS_SMALLBIG \
            -I$(GEN) -I$(SRC) -I$(SRC)/STUBS -I$(SRC)/MOLECULE -I$(SRC)/MANYBODY -I$(SRC)/USER-MISC
CFLAGS := -O2 -w -I$(SRC)/STUBS

CORE_CPP := $(filter-out $(SRC)/main.cpp,$(wildcard $(SRC)/*.cpp))
EXTRA_CPP := $(EXTRA)/atom_vec_ellipsoid.cpp $(EXTRA)/dihedral_hybrid.cpp $(EXTRA)/improper_hybrid.cpp
EXTRA_H := accelerator_kokkos.h accelerator_omp.h math_vector.h atom_vec_ellipsoid.h dihedral_hybrid.h improper_hybrid.h
PKG_CPP := $(wildcard $(SRC)/MOLECULE/*.cpp) $(SRC)/MANYBODY/pair_tersoff.cpp $(SRC)/USER-MISC/pair_ilp_graphene_hbn.cpp \
           $(SRC)/USER-MISC/pair_kolmogorov_crespi_full.cpp
ALL_CPP := $(CORE_CPP) $(EXTRA_CPP) $(PKG_CPP)
# headers of the compiled units: these (and only these) feed the style tables
STYLE_H := $(patsubst %.cpp,%.h,$(ALL_CPP))
OBJS := $(patsubst %.cpp,$(OBJ)/%.o,$(notdir $(ALL_CPP))) $(OBJ)/mpi.o

CLASSES := ANGLE:angle ATOM:atom BODY:body BOND:bond COMMAND:command COMPUTE:compute \
           DIHEDRAL:dihedral DUMP:dump FIX:fix IMPROPER:improper INTEGRATE:integrate \
           KSPACE:kspace MINIMIZE:minimize NBIN:nbin NPAIR:npair NSTENCIL:nstencil \
           NTOPO:ntopo PAIR:pair READER:reader REGION:region

all: $(OUT)/lmff_ref

$(GEN)/.stamp:
	@mkdir -p $(GEN) $(OBJ)
	@for h in $(EXTRA_H); do ln -sf $(EXTRA)/$$h $(GEN)/$$h; done
	@for c in $(CLASSES); do \
	   cls=$${c%%:*}; name=$${c##*:}; : > $(GEN)/style_$$name.h; : > $(GEN)/packages_$$name.h; \
	   for h in $(STYLE_H); do \
	     if [ -f $$h ] && grep -q "$${cls}_CLASS" $$h; then echo "#include \"$$(basename $$h)\"" >> $(GEN)/style_$$name.h; fi; \
	   done; \
	 done
	@printf '#ifndef LMP_INSTALLED_PKGS_H\n#define LMP_INSTALLED_PKGS_H\nconst char * LAMMPS_NS::LAMMPS::installed_packages[] = {"MANYBODY","MOLECULE","USER-MISC", NULL };\n#endif\n' > $(GEN)/lmpinstalledpkgs.h
	@printf '#ifndef LMP_GIT_VERSION_H\n#define LMP_GIT_VERSION_H\nconst bool LAMMPS_NS::LAMMPS::has_git_info = false;\nconst char LAMMPS_NS::LAMMPS::git_commit[] = "(unknown)";\nconst char LAMMPS_NS::LAMMPS::git_branch[] = "(unknown)";\nconst char LAMMPS_NS::LAMMPS::git_descriptor[] = "(unknown)";\n#endif\n' > $(GEN)/lmpgitversion.h
	@touch $@

vpath %.cpp $(SRC) $(SRC)/MOLECULE $(SRC)/MANYBODY $(SRC)/USER-MISC $(EXTRA)

$(OBJ)/%.o: %.cpp $(GEN)/.stamp
	@$(CXX) $(CXXFLAGS) -c $< -o $@

$(OBJ)/mpi.o: $(SRC)/STUBS/mpi.c $(GEN)/.stamp
	@$(CC) $(CFLAGS) -c $< -o $@

$(OBJ)/ref_harness.o: oracle/ref_harness.cpp $(GEN)/.stamp
	@$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/lmff_ref: $(OBJS) $(OBJ)/ref_harness.o
	@$(CXX) -o $@ $^ -lm

.PHONY: all

# ---------------------------------------------------------------------------------
# lmp_gb300: the same reference LAMMPS with the GB300 package's pair styles
# (lammps-lmff_gb300/lammps) registered, linked against liblmff_gb300.so.  Only the
# two core files that include the pair-style table (force.cpp, lammps.cpp) are
# recompiled with a table that adds the package's headers.  Used by the CPU test of
# the drop-in wiring (tests/test_lammps_package.py); the package itself is product code.
PKGDIR := lammps-lmff_gb300/lammps
GEN2 := $(OUT)/gen_gb300
OBJ2 := $(OUT)/obj_gb300
LIBDIR := lammps-lmff_gb300/lmff_gb300
PKG_SRC := $(PKGDIR)/pair_tersoff_gb300.cpp $(PKGDIR)/pair_ilp_graphene_hbn_gb300.cpp \
           $(PKGDIR)/pair_kolmogorov_crespi_full_gb300.cpp $(PKGDIR)/lmff_lammps_adapter.cpp \
           $(PKGDIR)/gb300_common.cpp
CXXFLAGS2 := -O2 -std=c++11 -w -ffp-contract=off -DLAMMPS_MEMALIGN=64 -DLAMMPS_SMALLBIG \
             -I$(GEN2) -I$(GEN) -I$(SRC) -I$(SRC)/STUBS -I$(SRC)/MOLECULE -I$(SRC)/MANYBODY -I$(SRC)/USER-MISC \
             -I$(PKGDIR) -Iinclude

$(GEN2)/style_pair.h: $(GEN)/.stamp
	@mkdir -p $(GEN2) $(OBJ2)
	@cp $(GEN)/style_pair.h $@
	@echo '#include "pair_tersoff_gb300.h"' >> $@
	@echo '#include "pair_ilp_graphene_hbn_gb300.h"' >> $@
	@echo '#include "pair_kolmogorov_crespi_full_gb300.h"' >> $@

$(OBJ2)/%.o: $(PKGDIR)/%.cpp $(GEN2)/style_pair.h
	@$(CXX) $(CXXFLAGS2) -c $< -o $@

$(OBJ2)/force.o: $(SRC)/force.cpp $(GEN2)/style_pair.h
	@$(CXX) $(CXXFLAGS2) -c $< -o $@

$(OBJ2)/lammps.o: $(SRC)/lammps.cpp $(GEN2)/style_pair.h
	@$(CXX) $(CXXFLAGS2) -c $< -o $@

$(OUT)/lmp_gb300: $(filter-out $(OBJ)/force.o $(OBJ)/lammps.o $(OBJ)/ref_harness.o,$(OBJS)) $(OBJ2)/force.o \
                  $(OBJ2)/lammps.o $(OBJ)/ref_harness.o $(patsubst $(PKGDIR)/%.cpp,$(OBJ2)/%.o,$(PKG_SRC))
	@$(CXX) -o $@ $^ -L$(LIBDIR) -llmff_gb300 -Wl,-rpath,$(abspath $(LIBDIR)) -lm

gb300: $(OUT)/lmp_gb300
.PHONY: gb300
