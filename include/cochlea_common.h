/*
 * cochlea_common.h -- the reference-named host API of the cochlear solver
 * path, served by libcochlea_gb300.so.
 *
 * Each declaration keeps the name, parameter list and C linkage of the
 * reference interface it replaces (YonatanKoral/CochlearModel,
 * include/cochlea_common.h:85-418, implemented there in src/cochlea.cu), so a
 * caller compiled against either header links against this library.  The
 * MSVC dynamic exception specification throw(...) is dropped; as in the
 * reference, failures raise std::runtime_error.  Device memory is owned by
 * the library (allocated by the *_Init / *NewKernel calls, released by the
 * *_Free calls); host pointers are borrowed for the duration of a call; every
 * call returns with its GPU work complete.
 *
 * Log is the caller's logger class (the reference's include/Log.h); the
 * library takes it by reference and never dereferences it.
 */
#ifndef COCHLEA_COMMON_H
#define COCHLEA_COMMON_H

#include <cuda_runtime.h>

#include <string>

#ifndef LAMBDA_COUNT
#define LAMBDA_COUNT 3
#endif

typedef float JNDFloat;
typedef float lambdaFloat;
class Log;

/* include/cochlea_common.h:31-49 */
typedef struct device_params_structs {
  int filter_b_start_index;
  int filter_a_start_index;
  int cochlea_sections;
  int calcTime;
  int writeTime;
  int time_blocks;
  int order_of_dc_filter;
  int order_of_ac_filter;
  int lambda_count;
  int time_block;
  int lambda_offset;
  int ovelapNodes;
  int FilterDecoupledMode;
  double Lambda_SAT;
  int intervalTimeNodes;
  float reverseSQRTScaleBMVelocityForLambdaCalculation;
  int Decouple_Filter;
} device_params;

/* include/cochlea_common.h:50-54 */
typedef struct vectors_sum_linear_coefficents_type {
  double A_coefficent;
  double B_coefficent;
  int reverseCoefficents;
} vectors_sum_linear_coefficents;

/* include/cochlea_common.h:56-66 */
typedef struct device_jnd_params_structs {
  double dA;
  double recipdA;
  double dBSPLSignal;
  double dBSPLNoise;
  double Wn;
  bool isReference;
  int calculateIndexPosition;
  int referenceIndex;
  double frequency;
} device_jnd_params;

#ifdef __cplusplus
extern "C" {
#endif

/* timing: include/cochlea_common.h:94-97 */
void cudaEventsCreate(cudaEvent_t& start, cudaEvent_t& stop, int condition);
void cudaEventsStartTimer(cudaEvent_t& start, cudaEvent_t& stop, int condition);
void cudaEventsStopTimer(cudaEvent_t& start, cudaEvent_t& stop, int condition);
float cudaEventsStopQueryTimer(cudaEvent_t& start, cudaEvent_t& stop, int condition,
                               const std::string& prefix);
/* buffers: include/cochlea_common.h:98-107 */
JNDFloat* getCudaBuffer();
JNDFloat* getCudaLambda();
void loadAihc(float* Aihc);
void enableloadAihc();
void allocateBuffer(const int size_in_nodes, int Show_Run_Time, cudaEvent_t& start,
                    cudaEvent_t& stop, cudaDeviceProp deviceProp);
void releaseBuffer(int Show_Run_Time, cudaEvent_t& start, cudaEvent_t& stop,
                   cudaDeviceProp deviceProp);

/* BM/OHC solver: include/cochlea_common.h:126-176 */
void BMOHCNewKernel(float* input_samples, bool override_input_samples, float w_ohc,
                    float time_step, float time_step_out, float delta_x, float alpha_r,
                    int enable_psi, int enable_OW, int base_index, float Ts, float _ohc_alpha_l,
                    float _ohc_alpha_s, float model_Gme, float model_a0, float model_a1,
                    float model_a2, float sigma_ow, float eta_1, float eta_2, float* tres,
                    int Time_Blocks, int samplesBufferLengthP1, int overlap_nodes_for_block,
                    long overlapTimeMicroSec, int show_transient, float cuda_max_time_step,
                    float cuda_min_time_step, int Decouple_Filter,
                    float Max_M1_SP_Error_Parameter, float Max_Tolerance_Parameter,
                    int Relative_Error_Parameters, int calculate_boundary_conditions,
                    float M1_SP_Fix_Factor, float Tolerance_Fix_Factor, float SPLREfVal,
                    int Show_Calculated_Power, int Show_Device_Data, int Show_Run_Time,
                    int JACOBBY_Loops_Fast, int JACOBBY_Loops_Slow, int Cuda_Outern_Loops,
                    int Run_Fast_BM_Calculation, int BMOHC_Kernel_Configuration,
                    cudaEvent_t& start, cudaEvent_t& stop, cudaDeviceProp deviceProp,
                    Log& outer_log);
/* include/cochlea_common.h:179-181 */
void BMOHCKernel_Wait_Threads();
void BMOHCKernel_Copy_Results(float* target, size_t resultNodes, size_t offset);
void extractConvergenceTimes(float* convergence_times, size_t nodes);

#ifdef __cplusplus
}
#endif

/* include/cochlea_common.h:186-191 (explicit instantiations for float,
 * double and int; updateCUDALambdaArray for float and double) */
template <class T>
extern void GeneralKernel_Copy_Results_Template(T* target, T* src, size_t size);
template <class T>
extern void GeneralKernel_Copy_Results_Template(T* target, T* src, size_t size, size_t offset);
template <class T>
extern void ReverseKernel_Copy_Results_Template(T* cpu_src, T* cuda_target,
                                                size_t start_time_node, size_t time_nodes,
                                                int sections);
template <class T>
extern void updateCUDALambdaArray(T* lambda_array, T* cuda_buffer, size_t calc_time_nodes,
                                  int sections, int Show_Run_Time, int Show_Device_Data,
                                  int cuda_buffer_update, Log& outer_log);

#ifdef __cplusplus
extern "C" {
#endif

/* include/cochlea_common.h:202-230 */
JNDFloat* getCudaMeanRate();
void GeneralKernel_Copy_Results(float* target, float* src, size_t size);
void GeneralKernel_Copy_Results_Double(double* target, double* src, size_t size);
void ReverseKernel_Copy_Results(float* src, size_t size);
void BMOHCKernel_Copy_Lambda(JNDFloat* target, size_t lambdaNodes, int offset);
void BMOHCKernel_Init(float* gamma, float* mass, float* M, float* U, float* L, float* R,
                      float* S, float* Q, float* S_ohc, float* S_tm, float* R_tm,
                      float num_frequencies, float dbA, size_t inputBufferNodes,
                      size_t resultBufferNodes, size_t lambdaBufferNodes, bool first_time,
                      int Show_Run_Time, int Show_Device_Data, Log& outer_log);

/* IHC / lambda: include/cochlea_common.h:237-280 */
void IHCNewKernel(double* IHC_Damage_Factor, float Nerves_Clusters[3 * LAMBDA_COUNT],
                  double* dc_filter, int order_of_dc_filter, double* ac_b_filter,
                  double* ac_a_filter, bool is_ac_iir_filter, int order_of_ac_filter,
                  int cochlea_sections, int time_blocks, double SPLRefVal, float* backup_speeds,
                  int backup_speeds_length, int calcTime, int writeTime, int allocateTime,
                  int intervalTimeNodes, int max_backup_nodes_len, int lambda_offset,
                  float Lambda_SAT, float eta_AC, float eta_DC, bool first_time,
                  bool first_time_for_param_set, bool loadedFromHD,
                  bool disable_advanced_memory_handling, bool review_memory_handling,
                  bool asMemoryHandlingOnly, float scaleBMVelocityForLambdaCalculation,
                  bool CalculateJNDOnGPU, int maxJNDIntervals, int overlapNodes,
                  int Decouple_Filter, int Show_Run_Time, Log& outer_log);
void RunIHCKernel(JNDFloat* host_backup, int Show_Run_Time, int save_lambda, int backup_stage,
                  int Decouple_Unified_IHC_Factor, Log& outer_log);
void cudaMallocatingByMode(void** ptr, size_t bytes_num, bool disable_advanced_mode);
void IHCKernel_Free();
void BMOHCKernel_Free();

/* input generation: include/cochlea_common.h:285-294, 365-417 */
void InputProfilesArrayInitialization(int maxJNDIntervals, int wn_length, int signal_length,
                                      int signal_mode, int Show_Generated_Input);
void viewGPUStatus(int flags, const std::string& prefix);
void InputProfilesArrayTermination();

/* JND: include/cochlea_common.h:296-331 */
void CudaCalculateJND(bool calculate_ai, bool calculate_rms, int mean_size, int fisher_size,
                      double SPLRefVal, double Fs, double scaleBMVelocityForLambdaCalculation,
                      double* nIHC, int* JND_Calculated_Intervals, int numOFJNDCalculated,
                      int* JND_Refrence_Intervals, int numOFJNDReferences,
                      int handeledIntervalsJND, int JNDIntervalsFull, int JNDIntervals,
                      int JNDIntervalHeadNodes, int overlapNodes, int JNDIntervalNodes,
                      int lengthOffset, int* JND_Serial_Intervals_Positions,
                      int* JND_Interval_To_Reference, JNDFloat* F_RA, JNDFloat* FisherAISum,
                      int writeMatrixSize, int calculatedMatrixSize,
                      double JND_Delta_Alpha_Length_Factor,
                      int JND_USE_Spont_Base_Reference_Lambda, int Show_Run_Time, bool calcdA,
                      bool show_generated_input_params_cuda, int backup_stage, Log& outer_log);

/* include/cochlea_common.h:347-363 */
void setupToleranceProfile(device_jnd_params* profiles, bool is_first_time_for_parameters_set,
                           float Max_M1_SP_Error_Parameter, float Max_Tolerance_Parameter,
                           int Relative_Error_Parameters, float M1_SP_Fix_Factor,
                           float Tolerance_Fix_Factor, int Blocks_Per_Interval,
                           int from_profile_index, int calculatedProfiles);
void uploadProfiles(device_jnd_params* profiles, int numOfProfiles, bool profilesLoaded);

/* include/cochlea_common.h:365-371 */
int* getCudaFailedTimeNodes();
int* getCudaFailedBlocks();
float* getCudaConvergeSpeedBlocks();
float* getCudaConvergedTimeNodes();
float* getCudaConvergedBlocks();
float* getCudaConvergedJacobyLoopsPerIteration();
float* getCudaConvergedJacobyLoopsPerIterationBlocks();

/* include/cochlea_common.h:375-417 */
void generateInputFromProfile(
    device_jnd_params* profiles, float* WN, int wn_length, float* Signal, int signal_length,
    int signal_mode, int Normalize_Sigma_Type, int Normalize_Sigma_Type_Signal,
    double Normalize_Noise_Energy_To_Given_Interval, double Remove_Generated_Noise_DC,
    int start_dc_expected_value_calculation, int end_dc_expected_value_calculation,
    int start_dc_normalized_value_calculation, int end_dc_normalized_value_calculation,
    int numOfProfiles, bool profilesLoaded, int from_profile_index, int calculatedProfiles,
    int overlapNodes, int IntervalLength, int JND_Interval_Head, int JND_Interval_Actual_Length,
    float Fs, int Show_Generated_Input, float* target_input, bool Show_Generated_Configuration,
    bool is_first_time_for_parameters_set, float Max_M1_SP_Error_Parameter,
    float Max_Tolerance_Parameter, int Relative_Error_Parameters, float M1_SP_Fix_Factor,
    float Tolerance_Fix_Factor, int Blocks_Per_Interval, int Show_Run_Time,
    float* fir_transfer_function, int fir_transfer_function_length,
    float* iir_transfer_function, int iir_transfer_function_length, Log& outer_log);

/* not in the reference header; defined in src/cochlea.cu:919-963 */
void calculateBoundariesForNonGeneratedInput(int Relative_Error_Parameters, int max_block_length,
                                             int Show_Calculated_Power, float M1_SP_Fix_Factor,
                                             float Tolerance_Fix_Factor,
                                             float Max_M1_SP_Error_Parameter,
                                             float Max_Tolerance_Parameter, float rSPLRefVal,
                                             int block_size, dim3 inputBlockDivision);

#ifdef __cplusplus
}
#endif

#endif /* COCHLEA_COMMON_H */
