# Builds oracle/_ref/libtdag_ref.so: the reference's own Transform-DAG sources, compiled where they
# lie under $(REF), plus ref_driver.cpp (C entry points) and the self-written stand-in headers of
# ref_shim/ for glm, libmorton, robin_hood, spdlog, fmt, TBB (serial), mio and nlohmann::json.
# Test infrastructure only; it needs the reference's sources, so it is built only where they exist.
#
# GCC 13 rejects three constructs that MSVC and Clang accept. They are rewritten by sed into
# equivalent forms, in copies under oracle/_ref/patched/ (never committed):
#  * large_sub_grid.h:148 and transform_dag.cpp:208 read a static constexpr member through a reference
#    parameter inside `if constexpr` (P2280, implemented in GCC 14): `x.subGridLevel` becomes the same
#    member named through the type;
#  * structure.h:253,275 import a dependent base-class type without `typename`.
# -I- stops quote includes from searching the including file's own directory, so the patched copies
# replace the originals for every includer; the other directories are listed with -iquote.
# transform_dag_hierarchical.cpp:750-751 explicitly instantiate an overload whose definition takes an
# rvalue reference; -fpermissive lets that through (the driver calls the four-argument overload).
REF ?= /root/reference
CXX ?= g++
HERE := $(dir $(abspath $(lastword $(MAKEFILE_LIST))))
OUT := $(HERE)_ref
PATCHED := $(OUT)/patched
T := $(REF)/tools
# libstdc++'s parallel-algorithm headers include each other with quotes, so -I- needs their directory.
PSTL := $(firstword $(wildcard $(addsuffix /pstl,$(shell $(CXX) -xc++ -E -v /dev/null 2>&1 | sed -n 's/^ \(\/.*\)/\1/p'))))

INC := -iquote $(PATCHED)/voxcom/voxel -iquote $(PATCHED) -I- -I $(HERE)ref_shim -I $(PATCHED) -I $(T)/lib/include \
       -iquote $(T)/lib/include/voxcom/voxel -iquote $(T)/lib/include/voxcom/utility -iquote $(T)/lib/include \
       -iquote $(T)/svdag_encoding/src -iquote $(PSTL)
# find_translation.cpp uses AVX2 intrinsics: the library is built for this x86_64 host only.
CXXFLAGS := -std=c++20 -O3 -fPIC -w -fpermissive -mavx2 -mbmi2 -include cstdint $(INC)

SRCS := $(T)/lib/src/voxel/find_translation.cpp $(T)/lib/src/voxel/transform_dag_hierarchical.cpp \
        $(T)/svdag_encoding/src/transform_dag_encoding.cpp $(T)/svdag_encoding/src/huffman.cpp
OBJS := $(patsubst %.cpp,$(OUT)/%.o,$(notdir $(SRCS))) $(OUT)/transform_dag.o $(OUT)/ref_driver.o
SHIMS := $(shell find $(HERE)ref_shim -type f)
PATCHES := $(PATCHED)/voxcom/voxel/large_sub_grid.h $(PATCHED)/voxcom/voxel/structure.h $(PATCHED)/src/transform_dag.cpp

all: $(OUT)/libtdag_ref.so

$(PATCHED)/voxcom/voxel/large_sub_grid.h: $(T)/lib/include/voxcom/voxel/large_sub_grid.h
	@mkdir -p $(dir $@)
	sed 's/outStructure\.subGridLevel/voxcom::EditStructure<void, uint32_t>::subGridLevel/' $< > $@

$(PATCHED)/voxcom/voxel/structure.h: $(T)/lib/include/voxcom/voxel/structure.h
	@mkdir -p $(dir $@)
	sed 's/using ParentType::BasicType;/using typename ParentType::BasicType;/' $< > $@

$(PATCHED)/src/transform_dag.cpp: $(T)/lib/src/voxel/transform_dag.cpp
	@mkdir -p $(dir $@)
	sed 's/if constexpr (Level == inDag\.subGridLevel)/if constexpr (Level == std::remove_cvref_t<decltype(inDag)>::subGridLevel)/' $< > $@

$(OUT)/find_translation.o: $(T)/lib/src/voxel/find_translation.cpp $(PATCHES) $(SHIMS)
	$(CXX) $(CXXFLAGS) -c $< -o $@
$(OUT)/transform_dag_hierarchical.o: $(T)/lib/src/voxel/transform_dag_hierarchical.cpp $(PATCHES) $(SHIMS)
	$(CXX) $(CXXFLAGS) -c $< -o $@
$(OUT)/transform_dag_encoding.o: $(T)/svdag_encoding/src/transform_dag_encoding.cpp $(PATCHES) $(SHIMS)
	$(CXX) $(CXXFLAGS) -c $< -o $@
$(OUT)/huffman.o: $(T)/svdag_encoding/src/huffman.cpp $(PATCHES) $(SHIMS)
	$(CXX) $(CXXFLAGS) -c $< -o $@
$(OUT)/transform_dag.o: $(PATCHED)/src/transform_dag.cpp $(PATCHES) $(SHIMS)
	$(CXX) $(CXXFLAGS) -c $< -o $@
$(OUT)/ref_driver.o: $(HERE)ref_driver.cpp $(PATCHES) $(SHIMS)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libtdag_ref.so: $(OBJS)
	$(CXX) -shared -o $@ $^

clean:
	rm -rf $(OUT)

.PHONY: all clean
