# Builds the reference's own CUDA sources (a staged copy, see build_ref.sh)
# into binaries under oracle/_ref/.  Test infrastructure only.
#   make -f oracle/ref.mk SRC=oracle/_ref/src_zt OUT=oracle/_ref/zt
NVCC   ?= nvcc
ARCH   ?= -gencode arch=compute_103a,code=sm_103a
FLAGS  := -O3 -Xptxas -O3 $(ARCH) -include cstdint
LIBSRC := entities/arg_parser entities/addition entities/flip_set schemes/scheme_integer schemes/scheme_z2 utils/utils
OBJ    := $(addprefix $(OUT)/obj/,$(addsuffix .o,$(LIBSRC)))
FG     := $(OUT)/obj/entities/flip_graph.o
CM     := $(OUT)/obj/entities/complexity_minimizer.o
AR     := $(OUT)/obj/entities/scheme_additions_reducer.o

all: $(OUT)/flip_graph $(OUT)/complexity_minimizer $(OUT)/additions_reducer $(OUT)/ref_harness

$(OUT)/obj/%.o: $(SRC)/%.cu
	@mkdir -p $(dir $@)
	$(NVCC) $(FLAGS) -I$(SRC) -dc $< -o $@

$(OUT)/obj/harness.o: oracle/ref_harness.cu
	@mkdir -p $(dir $@)
	$(NVCC) $(FLAGS) -I$(SRC) -dc $< -o $@

$(OUT)/flip_graph: $(OBJ) $(FG) $(OUT)/obj/main_flip_graph.o
	$(NVCC) $(FLAGS) $^ -o $@
$(OUT)/complexity_minimizer: $(OBJ) $(CM) $(OUT)/obj/main_complexity_minimizer.o
	$(NVCC) $(FLAGS) $^ -o $@
$(OUT)/additions_reducer: $(OBJ) $(AR) $(OUT)/obj/main_additions_reducer.o
	$(NVCC) $(FLAGS) $^ -o $@
$(OUT)/ref_harness: $(OBJ) $(FG) $(CM) $(AR) $(OUT)/obj/harness.o
	$(NVCC) $(FLAGS) $^ -o $@
