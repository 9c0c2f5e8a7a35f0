# Compiles the reference's own assembly sources, unmodified and from where they lie, against the
# project-written stand-ins in refshim/ (TEST INFRASTRUCTURE ONLY), into _ref/libnlfem_ref.so.
# Usage: make -f ref.mk REF=<path of the reference checkout>
# Same flags as the CPU restatement: -ffp-contract=off keeps FP64 rounding identical to the
# reference's unfused arithmetic; OpenMP as in the reference's setup.py.
REF ?=
CXX ?= g++
CXXFLAGS ?= -O3 -fPIC -std=c++17 -ffp-contract=off -fno-fast-math -fopenmp -w
HERE := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
OUT := $(HERE)_ref
SRCS := Cassemble.cpp integration.cpp model.cpp MeshTypes.cpp mathhelpers.cpp
OBJS := $(addprefix $(OUT)/,$(SRCS:.cpp=.o)) $(OUT)/ref_driver.o
INC := -I$(HERE)refshim -I$(REF)/include -I$(REF)/src
SHIMS := $(wildcard $(HERE)refshim/*) $(wildcard $(HERE)refshim/CGAL/*)

all: $(OUT)/libnlfem_ref.so

$(OUT):
	mkdir -p $(OUT)

$(OUT)/%.o: $(REF)/src/%.cpp $(SHIMS) | $(OUT)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/ref_driver.o: $(HERE)ref_driver.cpp $(SHIMS) | $(OUT)
	$(CXX) $(CXXFLAGS) $(INC) -c $< -o $@

$(OUT)/libnlfem_ref.so: $(OBJS)
	$(CXX) $(CXXFLAGS) -shared -o $@ $^

clean:
	rm -rf $(OUT)

.PHONY: all clean
